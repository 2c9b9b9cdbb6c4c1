"""Learned stage-1 pilot and the fast path (no counterpart in the reference).

The fast path replaces the hard-thresholding stage with a small residual
convolution net (``csrc/pilotnet.cu``) and runs the Wiener stage in full on
its pilot:

1. ``PilotNet.forward``: BF16 tensor-core inference of the net on the noisy
   volume (Anscombe domain, residual output);
2. per-tile residual check: the Poisson deviance of the input against the
   pilot is compared with its expectation under Poisson noise at the pilot's
   mean; tiles whose excess deviance per voxel lies outside
   ``[EXCESS_LOW, excess_high]`` are recomputed with the plain
   hard-thresholding stage (on the tile plus a halo of search radius + block
   voxels) and pasted back.  ``excess_high`` is calibrated on the plain
   stage-1 pilots of the training volumes;
3. the Wiener stage on that pilot, with the stage-2 settings of
   ``FAST_STAGE2`` (reference step 4, the approximate Poisson sigma for every
   plane, matching by screening distances with a rescoring of the selected
   candidates by the cancellation-free ratio form of the deviance).

The net is trained on the GPU by its own forward and backward kernels
(``PilotNet.fit``) on pairs (noisy volume, plain stage-1 estimate) that the
plain method generates on seeded synthetic phantoms (``training_pairs``).
"""

from __future__ import annotations

import copy
import ctypes
import math
import os

import numpy as np

from . import _abi, phantoms
from .api import _torch, stage_device, stage_launch, stage_prepare
from .validation import resolve_profile

# Stage-2 settings of the fast path by dimensionality (everything else stays at
# the profile's values).  3-D: reference step 4 instead of 3 and the
# approximate Poisson sigma for every plane (k = 0); chosen by a sweep at
# 256^3 on three seeds, where the learned pilot plus these settings gained
# 0.044 to 0.09 dB over the plain path at 7.2x its speed.
FAST_STAGE2 = {
    3: dict(wiener_step=(4, 4, 4), k=0),
    2: dict(),
}
# matching precision of the fast Wiener stage: the screening form on the
# patch's even sub-lattice for every candidate, then the full screening form
# for the 4 K smallest and a ratio-form rescoring of the selection; on three 256^3
# seeds it was 11% faster than "approx" and 0.03-0.04 dB better
FAST_MATCH_PRECISION = "subsampled"


class PilotNet:
    """Residual 3x3(x3) conv net, FP32 master parameters on the GPU."""

    def __init__(self, ndim: int = 3, channels: int = 48, layers: int = 8, params=None, seed: int = 0,
                 device: str = "cuda"):
        torch = _torch()
        self.ndim, self.channels, self.layers = int(ndim), int(channels), int(layers)
        self.device = torch.device(device)
        n = ctypes.c_int64(0)
        _abi.check(_abi.lib().bmnd_pilotnet_param_count(ctypes.byref(self._desc(1, (8,) * self.ndim)),
                                                        ctypes.byref(n)))
        self.n_params = n.value
        if params is None:
            params = _init_params(self.ndim, self.channels, self.layers, seed)
        params = np.asarray(params, dtype=np.float32).ravel()
        if params.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {params.size}")
        self.params = torch.from_numpy(params.copy()).to(self.device)
        self._m = torch.zeros_like(self.params)
        self._v = torch.zeros_like(self.params)
        self._grad = torch.zeros_like(self.params)
        self._loss = torch.zeros(1, dtype=torch.float64, device=self.device)
        self._sumsq = torch.zeros(1, dtype=torch.float64, device=self.device)
        self.step = 0
        self._packed = None
        self._packed_version = -1
        self._version = 0
        self._ws = {}
        self._last_desc = {}
        self.excess_high = DEFAULT_EXCESS_HIGH

    # -- plumbing ----------------------------------------------------------
    def _desc(self, batch, shape):
        d = _abi.PilotNet()
        d.ndim, d.channels, d.layers, d.batch = self.ndim, self.channels, self.layers, int(batch)
        for i, s in enumerate(shape):
            d.shape[i] = int(s)
        return d

    def _stream(self):
        return int(_torch().cuda.current_stream(self.device).cuda_stream)

    def packed(self):
        """BF16 fragment-ordered weights, repacked after every parameter change."""
        torch = _torch()
        if self._packed is None:
            nb = ctypes.c_uint64(0)
            _abi.check(_abi.lib().bmnd_pilotnet_packed_bytes(ctypes.byref(self._desc(1, (8,) * self.ndim)),
                                                             ctypes.byref(nb)))
            self._packed = torch.empty(nb.value, dtype=torch.uint8, device=self.device)
        if self._packed_version != self._version:
            _abi.check(_abi.lib().bmnd_pilotnet_pack(ctypes.byref(self._desc(1, (8,) * self.ndim)),
                                                     self.params.data_ptr(), self._packed.data_ptr(),
                                                     self._stream()))
            self._packed_version = self._version
        return self._packed

    def _workspace(self, desc, training):
        torch = _torch()
        nb = ctypes.c_uint64(0)
        _abi.check(_abi.lib().bmnd_pilotnet_workspace_bytes(ctypes.byref(desc), int(training), ctypes.byref(nb)))
        key = bool(training)
        self._last_desc[key] = desc
        ws = self._ws.get(key)
        if ws is None or ws.numel() < nb.value:
            ws = torch.empty(nb.value, dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        return ws

    @staticmethod
    def _batched(x, ndim):
        if x.dim() == ndim:
            return x.unsqueeze(0), True
        if x.dim() == ndim + 1:
            return x, False
        raise ValueError(f"expected a {ndim}-D volume or a batch of them, got shape {tuple(x.shape)}")

    # -- inference ---------------------------------------------------------
    def forward(self, noisy, want_y: bool = False):
        """Pilot (count domain) of a float32 CUDA volume or batch of volumes."""
        torch = _torch()
        x, single = self._batched(noisy.contiguous().to(torch.float32), self.ndim)
        desc = self._desc(x.shape[0], x.shape[1:])
        ws = self._workspace(desc, False)
        pilot = torch.empty_like(x)
        y = torch.empty_like(x) if want_y else None
        _abi.check(_abi.lib().bmnd_pilotnet_forward(
            ctypes.byref(desc), self.packed().data_ptr(), x.data_ptr(), pilot.data_ptr(),
            None if y is None else y.data_ptr(), ws.data_ptr(), ws.numel(), self._stream()))
        if single:
            pilot = pilot[0]
            y = None if y is None else y[0]
        return (pilot, y) if want_y else pilot

    def check_status(self, training: bool = False) -> None:
        """Raise if a bounded tensor-core wait of the last forward (or, with
        ``training``, gradient) call ran out; synchronises the stream."""
        ws = self._ws.get(bool(training))
        if ws is None:
            return
        desc = self._last_desc.get(bool(training))
        _abi.check(_abi.lib().bmnd_pilotnet_status(ctypes.byref(desc), ws.data_ptr(), self._stream()))

    # -- training ----------------------------------------------------------
    def gradient(self, noisy, target):
        """(loss, gradient) of mean((y - A(target))^2) for a batch; the
        gradient tensor is reused by the next call."""
        torch = _torch()
        x, _ = self._batched(noisy.contiguous().to(torch.float32), self.ndim)
        t, _ = self._batched(target.contiguous().to(torch.float32), self.ndim)
        desc = self._desc(x.shape[0], x.shape[1:])
        ws = self._workspace(desc, True)
        _abi.check(_abi.lib().bmnd_pilotnet_gradient(
            ctypes.byref(desc), self.packed().data_ptr(), x.data_ptr(), t.data_ptr(), self._grad.data_ptr(),
            self._loss.data_ptr(), ws.data_ptr(), ws.numel(), self._stream()))
        return self._loss, self._grad

    def adam_step(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  clip: float = 1.0):
        """Adam on the last gradient, clipped to an L2 norm of ``clip`` (<= 0: none)."""
        self.step += 1
        _abi.check(_abi.lib().bmnd_pilotnet_adam(
            self.n_params, self.params.data_ptr(), self._grad.data_ptr(), self._m.data_ptr(), self._v.data_ptr(),
            self.step, float(lr), float(beta1), float(beta2), float(eps), float(clip), self._sumsq.data_ptr(),
            self._stream()))
        self._version += 1

    def fit(self, pairs, steps: int = 2000, crop: int = 32, batch: int = 4, lr: float = 3e-4, seed: int = 0,
            log_every: int = 100, log=None, clip: float = 1.0):
        """Adam on random crops of (noisy, target) CUDA volume pairs; returns the
        loss history.  The gradient is clipped to an L2 norm of ``clip``; the
        parameters with the lowest logged loss (a running mean over the last
        ``log_every`` steps) are kept at the end, which guards against a late
        divergence."""
        torch = _torch()
        rng = np.random.default_rng(seed)
        shape = tuple(int(s) for s in pairs[0][0].shape)
        cs = tuple(min(crop, s) for s in shape)
        xb = torch.empty((batch,) + cs, dtype=torch.float32, device=self.device)
        tb = torch.empty_like(xb)
        running = torch.zeros(1, dtype=torch.float64, device=self.device)
        best, best_params = math.inf, None
        history = []
        for it in range(steps):
            for b in range(batch):
                k = int(rng.integers(len(pairs)))
                x, t = pairs[k]
                o = [int(rng.integers(0, s - c + 1)) for s, c in zip(x.shape, cs)]
                sl = tuple(slice(a, a + c) for a, c in zip(o, cs))
                xb[b].copy_(x[sl])
                tb[b].copy_(t[sl])
            loss, _ = self.gradient(xb, tb)
            running += loss
            frac = it / max(steps - 1, 1)
            rate = lr * (0.5 * (1.0 + math.cos(math.pi * frac)) * 0.9 + 0.1)  # cosine to lr / 10
            self.adam_step(rate, clip=clip)
            if (it + 1) % log_every == 0 or it == steps - 1:
                n = (it % log_every) + 1
                value = float(running.item()) / n
                running.zero_()
                history.append((it + 1, value))
                if value < best:
                    best = value
                    best_params = self.params.clone()
                self.check_status(training=True)
                if log:
                    log(f"step {it + 1} loss {value:.6f} grad_norm {math.sqrt(float(self._sumsq.item())):.4f}")
        if best_params is not None:
            self.params.copy_(best_params)
            self._version += 1
        return history

    # -- persistence -------------------------------------------------------
    def state(self) -> dict:
        return dict(params=self.params.detach().cpu().numpy(), ndim=self.ndim, channels=self.channels,
                    layers=self.layers, excess_high=self.excess_high)

    def save(self, path: str) -> None:
        np.savez(path, **self.state())

    @classmethod
    def load(cls, path: str, device: str = "cuda") -> "PilotNet":
        d = np.load(path)
        net = cls(int(d["ndim"]), int(d["channels"]), int(d["layers"]), params=d["params"], device=device)
        if "excess_high" in d:
            net.excess_high = float(d["excess_high"])
        return net


def _init_params(ndim, channels, layers, seed, out_scale=0.1):
    """He-normal weights, zero biases; the residual branch starts small."""
    rng = np.random.default_rng(seed)
    taps = 3 ** ndim
    parts = []
    for l in range(layers):
        cin = 1 if l == 0 else channels
        cout = 1 if l == layers - 1 else channels
        std = math.sqrt(2.0 / (taps * cin)) * (out_scale if l == layers - 1 else 1.0)
        parts.append(rng.normal(0.0, std, size=taps * cin * cout))
        parts.append(np.zeros(cout))
    return np.concatenate(parts).astype(np.float32)


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def lowcount_peak(seed: int) -> float:
    """Peak count of the low-count 3-D phantoms: uniform in [2, 5], from the seed."""
    return float(np.random.default_rng(10_000 + seed).uniform(2.0, 5.0))


def training_pairs(kind: str = "bm4d", size: int = 128, count: int = 8, seed0: int = 1000, profile=None):
    """(noisy, plain stage-1 estimate) CUDA pairs on seeded phantoms (seeds
    seed0 .. seed0 + count - 1, disjoint from the benchmark's).  ``kind``
    "bm4d_lowcount" scales each ellipsoid volume to a peak of
    ``lowcount_peak(seed)`` counts; "bm3d_windows" takes ``size``-square
    windows of 2048^2 blob phantoms (``phantoms.blobs_2d_window``)."""
    torch = _torch()
    import bmnd_gb300 as bg

    if profile is None:
        profile = (bg.BM3DProfile if kind.startswith("bm3d") else bg.BM4DProfile)(noise_model=bg.NoiseModel.POISSON)
    pairs = []
    for i in range(count):
        if kind == "bm3d_windows":
            _, noisy = phantoms.blobs_2d_window(size, seed=seed0 + i)
        elif kind == "bm4d_lowcount":
            _, noisy = phantoms.ellipsoids_3d(size, seed=seed0 + i, peak=lowcount_peak(seed0 + i))
        elif kind == "bm4d":
            _, noisy = phantoms.ellipsoids_3d(size, seed=seed0 + i)
        elif size >= 1024:
            _, noisy = phantoms.blobs_2d(size, seed=seed0 + i)
        else:
            _, noisy = phantoms.shapes_2d(size, seed=seed0 + i)
        x = torch.from_numpy(noisy).cuda()
        pairs.append((x, stage_device(x, profile, "ht")))
    return pairs


# ---------------------------------------------------------------------------
# per-tile residual check and fallback
# ---------------------------------------------------------------------------
_TABLE = None


def deviance_table(n: int = 512, mu_min: float = 1e-3, mu_max: float = 1e4):
    """Expectation and variance of the Poisson unit deviance 2 [x ln(x/mu) - (x - mu)]
    for x ~ Poisson(mu), on a log grid of mu (summed over the pmf)."""
    from math import lgamma

    mus = np.exp(np.linspace(math.log(mu_min), math.log(mu_max), n))
    ev = np.empty(n)
    vv = np.empty(n)
    for i, mu in enumerate(mus):
        hi = int(mu + 12.0 * math.sqrt(mu) + 40)
        x = np.arange(hi + 1, dtype=np.float64)
        logp = x * math.log(mu) - mu - np.array([lgamma(k + 1.0) for k in x])
        p = np.exp(logp)
        with np.errstate(divide="ignore", invalid="ignore"):
            d = 2.0 * (np.where(x > 0, x * np.log(np.where(x > 0, x, 1.0) / mu), 0.0) - (x - mu))
        e = float(np.sum(p * d))
        ev[i] = e
        vv[i] = float(np.sum(p * d * d)) - e * e
    return mus, ev, vv


def _device_table(device):
    global _TABLE
    torch = _torch()
    if _TABLE is None:
        mus, ev, vv = deviance_table()
        _TABLE = (np.concatenate([ev, vv]).astype(np.float32), float(np.log(mus[0])),
                  float(np.log(mus[1]) - np.log(mus[0])), len(mus))
    data, ln0, dln, n = _TABLE
    return torch.from_numpy(data).to(device), ln0, dln, n


def tile_stats(noisy, pilot, edge: int):
    """Per tile (x fastest, then y, z): observed deviance, its expectation and
    variance under Poisson noise at the pilot, and the voxel count."""
    torch = _torch()
    nd = noisy.dim()
    shape = tuple(int(s) for s in noisy.shape)
    grid = tuple((s + edge - 1) // edge for s in shape)
    ntiles = int(np.prod(grid))
    out = torch.empty((ntiles, 3), dtype=torch.float64, device=noisy.device)
    table, ln0, dln, n = _device_table(noisy.device)
    sh = (ctypes.c_int32 * nd)(*shape)
    _abi.check(_abi.lib().bmnd_pilot_tile_deviance(
        nd, 1, sh, int(edge), noisy.data_ptr(), pilot.data_ptr(), table.data_ptr(), n, ln0, dln, out.data_ptr(),
        int(torch.cuda.current_stream(noisy.device).cuda_stream)))
    s = out.cpu().numpy()
    counts = np.ones(grid, dtype=np.float64)
    for d in range(nd):
        ext = np.full(grid[d], float(edge))
        ext[-1] = shape[d] - edge * (grid[d] - 1)
        counts = counts * ext.reshape([-1 if i == d else 1 for i in range(nd)])
    # reverse so that the last (x) axis varies fastest, as the kernel orders tiles
    return s[:, 0].reshape(grid), s[:, 1].reshape(grid), s[:, 2].reshape(grid), counts, grid


def tile_zscores(noisy, pilot, edge: int):
    """Standardised excess deviance (observed - expected) / sqrt(variance) per tile."""
    obs, exp, var, _, grid = tile_stats(noisy, pilot, edge)
    return (obs - exp) / np.sqrt(np.maximum(var, 1e-12)), grid


def tile_excess(noisy, pilot, edge: int):
    """Excess deviance per voxel, (observed - expected) / voxels, per tile."""
    obs, exp, _, counts, grid = tile_stats(noisy, pilot, edge)
    return (obs - exp) / counts, grid


def apply_fallback(noisy, pilot, profile, fail, edge: int):
    """Recompute the tiles flagged in ``fail`` with the plain stage 1 (on the
    tile plus a halo of search radius + block) and paste them into ``pilot``;
    returns the count."""
    nd = noisy.dim()
    shape = tuple(int(s) for s in noisy.shape)
    block = tuple(int(b) for b in profile.ht_block_size)
    radius = tuple(int(r) for r in profile.ht_search_window)
    halo = tuple(r + b for r, b in zip(radius, block))
    bad = np.argwhere(fail)
    for t in bad:
        lo = [int(t[d]) * edge for d in range(nd)]
        hi = [min(lo[d] + edge, shape[d]) for d in range(nd)]
        clo = [max(lo[d] - halo[d], 0) for d in range(nd)]
        chi = [min(hi[d] + halo[d], shape[d]) for d in range(nd)]
        crop = noisy[tuple(slice(a, b) for a, b in zip(clo, chi))].contiguous()
        if not bool((crop != 0).any()):
            est = crop.clone()
        else:
            est = stage_device(crop, profile, "ht")
        inner = tuple(slice(lo[d] - clo[d], hi[d] - clo[d]) for d in range(nd))
        pilot[tuple(slice(a, b) for a, b in zip(lo, hi))] = est[inner]
    return len(bad)


# the residual check: a tile falls back when its excess deviance per voxel lies
# outside [EXCESS_LOW, excess_high]; excess_high is calibrated per network on
# the plain stage-1 pilots of its training volumes (PilotNet.excess_high),
# EXCESS_LOW catches a pilot that follows the noise (the excess of the noisy
# input itself is about -1 per voxel)
EXCESS_LOW = -0.25
DEFAULT_EXCESS_HIGH = 0.5


# ---------------------------------------------------------------------------
# the fast path
# ---------------------------------------------------------------------------
def fast_profile(profile):
    """Copy of ``profile`` with the fast path's stage-2 settings."""
    p = copy.deepcopy(profile)
    for k, v in FAST_STAGE2[len(tuple(profile.wiener_block_size))].items():
        setattr(p, k, v)
    return p


_CONV_ENGINES = {"tcgen05": _abi.CONV_TCGEN05, "mma_sync": _abi.CONV_MMA_SYNC}


def set_conv_engine(name: str) -> None:
    """Engine of the pilot net's C -> C layers, process-wide: "tcgen05"
    (default; accumulator in tensor memory) or "mma_sync" (warp-level MMA)."""
    if name not in _CONV_ENGINES:
        raise ValueError(f"conv engine must be one of {sorted(_CONV_ENGINES)}")
    _abi.check(_abi.lib().bmnd_pilotnet_set_conv_engine(_CONV_ENGINES[name]))


def get_conv_engine() -> str:
    v = ctypes.c_int32(0)
    _abi.check(_abi.lib().bmnd_pilotnet_get_conv_engine(ctypes.byref(v)))
    return {c: n for n, c in _CONV_ENGINES.items()}[v.value]


def default_tile(ndim: int) -> int:
    """Residual-check tile edge: 32^3 voxels in 3-D, 64^2 pixels in 2-D."""
    return 32 if ndim == 3 else 64


def bmnd_fast(noisy, profile, net: PilotNet, *, tile: int | None = None, excess_high: float | None = None,
              stage2: bool = True, match_precision: str = FAST_MATCH_PRECISION, check: bool = True,
              details: dict | None = None):
    """Learned-pilot fast path on a float32 CUDA volume; returns the CUDA estimate.

    ``details`` (a dict, optional) receives the pilot, the per-tile excess
    deviance and the number of tiles that fell back to the plain stage 1."""
    torch = _torch()
    x = noisy.contiguous().to(torch.float32)
    shape = tuple(int(s) for s in x.shape)
    resolve_profile(profile, shape)
    if tile is None:
        tile = default_tile(x.dim())
    pilot = net.forward(x)
    # the Wiener stage's host-side preparation runs while the net is on the device
    p2 = fast_profile(profile) if stage2 else profile
    prep = stage_prepare(x, p2, "wiener", match_precision=match_precision if stage2 else "exact",
                         fast_transforms=stage2)
    n_fb, excess = 0, None
    if check:
        hi = excess_high if excess_high is not None else net.excess_high
        excess, _ = tile_excess(x, pilot, tile)
        net.check_status()
        fail = (excess > hi) | (excess < EXCESS_LOW)
        n_fb = apply_fallback(x, pilot, profile, fail, tile)
    if details is not None:
        details.update(pilot=pilot, excess=excess, fallback_tiles=n_fb,
                       tiles=int(np.prod([(s + tile - 1) // tile for s in shape])))
    return stage_launch(prep, x, pilot)


def calibrate_excess_high(pairs, tile: int | None = None, spread: float = 3.0) -> float:
    """Upper bound of the per-tile excess deviance: the largest value the plain
    stage-1 pilots (the training targets) reach on the training volumes, plus
    ``spread`` standard deviations of their per-tile values."""
    vals = []
    for x, t in pairs:
        e, _ = tile_excess(x, t, tile or default_tile(x.dim()))
        vals.append(np.ravel(e))
    v = np.concatenate(vals)
    return float(np.max(v) + spread * np.std(v))


def default_net_path(kind: str = "bm4d") -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", f"pilot_{kind}.npz")
