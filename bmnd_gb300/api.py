"""``bmnd()``: the reference's public entry point, executed on one GB300.

Same signature, argument checks (in the same order, with the same
``ValueError`` texts), return contract and callbacks as the reference
(src/bmnd/bmndalgo.py:71-183, :325-326, :632-633, :742-743, :1045-1046).
Below the validation every step runs in the native library
(``libbmnd_gb300.so``) on the current CUDA device; PyTorch only provides the
device buffers and the stream.  There is no CPU fallback: without a CUDA
device, or without the built library, the call raises.

Scope of the GPU path: direct-Poisson profiles (``noise_model="poisson"``)
with the default Poisson options, and stationary Gaussian noise
(``noise_model="gaussian"``, with ``sigma``, a ``sigma_psd`` or neither, in
which case sigma is estimated), on 1-3 dimensional volumes with patch edges up
to 8 and stacks up to 32.  Anything else raises ``NotImplementedError`` after
validation.
"""

from __future__ import annotations

import ctypes
import threading
from collections.abc import Callable
from dataclasses import dataclass

import numpy as np

from . import _abi, gaussian, plan, policies
from .enums import BlockMatchDistance, CacheMode, coerce_enum
from .validation import resolve_profile

__all__ = ["bmnd", "BlockMatchGroup", "BlockMatchResult", "bmnd_device", "group_probe"]


@dataclass
class BlockMatchGroup:
    """One matched group, as the reference reports it (blockmatching.py:151-160)."""

    reference_abs: tuple[int, ...]
    reference_shift: tuple[int, ...]
    reference_shifted: tuple[int, ...]
    selected_lin_indices: np.ndarray
    selected_abs_positions: np.ndarray
    selected_shifted_positions: np.ndarray
    accepted_count: int
    final_count: int


@dataclass
class BlockMatchResult:
    groups: list[BlockMatchGroup]


def _validate_sigma(sigma: object) -> float:
    if isinstance(sigma, (bool, np.bool_)):
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.")
    try:
        value = float(sigma)
    except (TypeError, ValueError) as exc:
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.") from exc
    if not np.isfinite(value) or value < 0.0:
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.")
    return value


def _validate_max_cache_bytes(budget):
    """Same accepted values as the reference (cache.py:65-83); the budget itself
    governs CPU-side covariance caches the GPU path does not have."""
    if isinstance(budget, str):
        budget = coerce_enum(budget, CacheMode, "max_cache_bytes mode")
    if budget is None or budget is CacheMode.AUTO:
        return budget
    if isinstance(budget, bool) or not isinstance(budget, (int, np.integer)) or int(budget) < 0:
        raise ValueError(
            "max_cache_bytes must be a non-negative integer, 'auto', or None, "
            f"got {budget!r}."
        )
    return int(budget)


def _torch():
    import torch

    return torch


class _Workspace:
    """Per-device scratch buffer, grown on demand and reused across calls."""

    def __init__(self):
        self._lock = threading.Lock()
        self._buffers = {}

    def get(self, device, nbytes: int):
        torch = _torch()
        key = str(device)
        with self._lock:
            buf = self._buffers.get(key)
            if buf is None or buf.numel() < nbytes:
                buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
                if buf.data_ptr() % 256:
                    raise RuntimeError("workspace allocation is not 256-byte aligned")
                self._buffers[key] = buf
            return buf


_WORKSPACE = _Workspace()
_REFS_CACHE: dict = {}


class _Staging:
    """Host <-> device transfers of the NumPy path of :func:`bmnd`.

    Where the device reads ordinary host memory through the host's page
    tables (a Grace host over NVLink-C2C), the arrays are copied directly: a
    64 MiB transfer then takes about 0.4 ms either way, the rate of a
    page-locked one.  Elsewhere page-locked host buffers, grown on demand and
    reused, carry the data: the input is copied into one and sent to the
    device asynchronously, the result comes back through the other.  The
    host-side copies are split over a few threads (NumPy releases the
    interpreter lock while it copies), and the upload goes in slices, each
    slice's transfer overlapping the copy of the next.  A lock makes
    concurrent host threads take turns."""

    _SLICES = 8

    def __init__(self):
        self._lock = threading.Lock()
        self._bufs = {}
        self._pool = None
        self._direct = {}

    def _is_direct(self, device: int) -> bool:
        d = self._direct.get(device)
        if d is None:
            d = self._direct[device] = _abi.host_memory_direct(device)
        return d

    def _get(self, key, numel):
        torch = _torch()
        buf = self._bufs.get(key)
        if buf is None or buf.numel() < numel:
            buf = torch.empty(max(int(numel), 1), dtype=torch.float32).pin_memory()
            self._bufs[key] = buf
        return buf[:numel]

    def _threads(self):
        if self._pool is None:
            import os
            from concurrent.futures import ThreadPoolExecutor

            self._pool = ThreadPoolExecutor(max(1, min(8, os.cpu_count() or 1)), thread_name_prefix="bmnd-copy")
        return self._pool

    def _copy(self, dst: np.ndarray, src: np.ndarray) -> None:
        """dst[...] = src over flat float32 arrays, in parallel slices."""
        n = src.size
        if n < (1 << 20):
            np.copyto(dst, src)
            return
        parts = self._SLICES
        step = (n + parts - 1) // parts
        list(self._threads().map(lambda i: np.copyto(dst[i * step:(i + 1) * step], src[i * step:(i + 1) * step]),
                                 range(parts)))

    def upload(self, arr: np.ndarray):
        torch = _torch()
        device = torch.cuda.current_device()
        if self._is_direct(device):
            dev = torch.empty(arr.shape, dtype=torch.float32, device=device)
            dev.copy_(torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32)))
            return dev
        with self._lock:
            flat = arr.reshape(-1)
            host = self._get("in", flat.size)
            dev = torch.empty(arr.shape, dtype=torch.float32, device=torch.cuda.current_device())
            dflat = dev.view(-1)
            n = flat.size
            parts = self._SLICES if n >= (1 << 22) else 1
            step = (n + parts - 1) // parts
            hnp = host.numpy()
            for i in range(parts):
                lo, hi = i * step, min(n, (i + 1) * step)
                if lo >= hi:
                    break
                self._copy(hnp[lo:hi], flat[lo:hi])
                dflat[lo:hi].copy_(host[lo:hi], non_blocking=True)
            # the staging buffer is reused by the next call: wait for the copies
            torch.cuda.current_stream().synchronize()
        return dev

    def result_buffer(self, shape):
        """A float32 host array of `shape` for a result that :meth:`download`
        will fill directly, with its pages touched on worker threads while the
        device computes (a fresh 64 MiB array otherwise takes about 3 ms of page
        faults inside the copy).  Returns a future of the array, or None where
        results go through the page-locked buffers."""
        torch = _torch()
        n = int(np.prod(shape)) if len(shape) else 1
        if n < (1 << 20) or not self._is_direct(torch.cuda.current_device()):
            return None
        out = np.empty(tuple(shape), dtype=np.float32)
        flat = out.reshape(-1)
        parts = self._SLICES
        step = (n + parts - 1) // parts
        pool = self._threads()
        futs = [pool.submit(flat[i * step:(i + 1) * step].fill, 0.0) for i in range(parts)]

        class _Ready:
            def result(self_inner):
                for f in futs:
                    f.result()
                return out

        return _Ready()

    def download(self, t, into=None) -> np.ndarray:
        torch = _torch()
        if self._is_direct(t.device.index if t.device.index is not None else torch.cuda.current_device()):
            out = into.result() if into is not None else np.empty(tuple(t.shape), dtype=np.float32)
            torch.from_numpy(out).copy_(t)
            return out
        with self._lock:
            flat = t.reshape(-1)
            n = flat.numel()
            host = self._get("out", n)
            out = np.empty(tuple(t.shape), dtype=np.float32)
            oflat = out.reshape(-1)
            hnp = host.numpy()
            parts = self._SLICES if n >= (1 << 22) else 1
            step = (n + parts - 1) // parts
            # every slice's transfer is queued behind an event, and each slice
            # is copied out on the host while the later ones are still in flight
            stream = torch.cuda.current_stream()
            events = []
            for i in range(parts):
                lo, hi = i * step, min(n, (i + 1) * step)
                if lo >= hi:
                    break
                host[lo:hi].copy_(flat[lo:hi], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(stream)
                events.append((lo, hi, ev))
            for lo, hi, ev in events:
                ev.synchronize()
                self._copy(oflat[lo:hi], hnp[lo:hi])
            return out


_STAGING = _Staging()
_CUDA_READY = None


def _cuda_ready() -> bool:
    """Whether a CUDA device is present (checked once)."""
    global _CUDA_READY
    if _CUDA_READY is None:
        _CUDA_READY = bool(_torch().cuda.is_available())
    return _CUDA_READY


def _host_result(t, into=None) -> np.ndarray:
    return _STAGING.download(t, into)


_NETS: dict = {}


def _learned_net(ndim: int, path: str | None, device):
    """The learned pilot's net for ``ndim``-D volumes, loaded once per file and device."""
    from . import pilot as pilot_mod

    if path is None:
        path = pilot_mod.default_net_path("bm4d" if ndim == 3 else "bm3d")
    key = (path, str(device))
    net = _NETS.get(key)
    if net is None:
        net = pilot_mod.PilotNet.load(path, device=str(device))
        if net.ndim != ndim:
            raise ValueError(f"pilot weights {path!r} are for {net.ndim}-D volumes, the input is {ndim}-D")
        _NETS[key] = net
    return net


def _device_refs(schedule: plan.Schedule, device):
    torch = _torch()
    key = (id(schedule), str(device))
    hit = _REFS_CACHE.get(key)
    if hit is not None and hit[0] is schedule:
        return hit[1]
    t = torch.from_numpy(np.array(schedule.reference_abs, dtype=np.int32, copy=True)).to(device)
    if len(_REFS_CACHE) > 64:
        _REFS_CACHE.clear()
    _REFS_CACHE[key] = (schedule, t)
    return t


def _match_result(schedule: plan.Schedule, counts, sel, cnt, acc) -> BlockMatchResult:
    ndim = len(counts)
    groups = []
    counts_arr = np.asarray(counts, dtype=np.int64)
    for i in range(len(schedule)):
        k = int(cnt[i])
        lins = sel[i, :k].astype(np.int64)
        abs_pos = np.stack(np.unravel_index(lins, counts_arr), axis=1).astype(np.int64) if k else np.empty(
            (0, ndim), dtype=np.int64
        )
        if k:
            shifted = abs_pos - abs_pos.min(axis=0, keepdims=True)
            ref_shifted = tuple(int(x) for x in shifted[0])
        else:
            shifted = abs_pos.copy()
            ref_shifted = tuple(int(x) for x in schedule.reference_shifted[i])
        groups.append(
            BlockMatchGroup(
                reference_abs=tuple(int(x) for x in schedule.reference_abs[i]),
                reference_shift=tuple(int(x) for x in schedule.shift[i]),
                reference_shifted=ref_shifted,
                selected_lin_indices=lins,
                selected_abs_positions=abs_pos,
                selected_shifted_positions=shifted,
                accepted_count=int(acc[i]),
                final_count=k,
            )
        )
    return BlockMatchResult(groups=groups)


_MATCH_PRECISIONS = {"exact": _abi.MATCH_EXACT, "fast": _abi.MATCH_FAST, "approx": _abi.MATCH_APPROX,
                     "subsampled": _abi.MATCH_SUBSAMPLED}


_NULL_TABLES: dict = {}


def null_table_device(profile, resolved, device):
    """The null moment table of the profile's Poisson HT match policy as a
    CUDA tensor, or None for the fixed policy (cached per device)."""
    from .enums import PoissonHTMatchPolicy

    if not resolved.is_poisson or profile.poisson_ht_match_policy is PoissonHTMatchPolicy.FIXED:
        return None
    key = (resolved.blockmatch_distance, int(profile.poisson_ht_match_moment_max_count), str(device))
    hit = _NULL_TABLES.get(key)
    if hit is None:
        table = policies.null_moment_table(key[0], key[1])
        hit = _torch().from_numpy(np.array(table, dtype=np.float64)).to(device)
        _NULL_TABLES[key] = hit
    return hit


def gaussian_tables(model: gaussian.GaussianModel, profile, shape, resolved, device) -> dict:
    """Device tables of both stages for stationary Gaussian noise: the
    covariance maps of each stage's transformed patches ([lag][coefficient])
    and, for hard thresholding with gamma != 0, the SSD noise bias over the
    search window (bmndalgo.py:291-303)."""
    torch = _torch()
    out = {}
    for stage in ("ht", "wiener"):
        block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
        maps = gaussian.covariance_maps(model, block, plan.spatial_forward(profile, len(shape), stage))
        cov = torch.from_numpy(np.ascontiguousarray(maps.reshape(maps.shape[0], -1).T)).to(device)
        entry = {"cov": cov, "domain": model.domain, "ssd": None, "gamma": 0.0,
                 "white_variance": gaussian.white_variance(model)}
        if stage == "ht" and resolved.blockmatch_distance is BlockMatchDistance.SSD:
            gamma = 0.0 if resolved.conventional_nf else float(profile.gamma)
            if gamma != 0.0:
                radius = tuple(int(r) for r in profile.ht_search_window)
                table = gaussian.blockmatch_noise_ssd(model, block, radius)
                entry["ssd"] = torch.from_numpy(np.ascontiguousarray(table.reshape(-1))).to(device)
                entry["gamma"] = float(np.float32(gamma))
        out[stage] = entry
    return out


def bmnd_device(noisy, profile, *, resolved=None, match_precision: str = "exact",
                stage_callback=None, blockmatch_callback=None, stream=None, sigma_maps: dict | None = None,
                global_sigma: float = 0.0, gauss: dict | None = None):
    """Run both stages on a float32 CUDA tensor and return the CUDA result tensor.

    ``noisy`` must be a C-contiguous float32 CUDA tensor holding a validated,
    non-negative, non-zero volume.  This is the device-resident core of
    :func:`bmnd` (no host copies unless a callback is given).  With a
    ``sigma_maps`` dict, each stage also writes its sigma map (CUDA tensor,
    keys "ht" and "wiener"; uncovered voxels get ``global_sigma``).  ``gauss``
    (from :func:`gaussian_tables`) selects stationary Gaussian noise.
    """
    torch = _torch()
    shape = tuple(int(s) for s in noisy.shape)
    if resolved is None:
        resolved = resolve_profile(profile, shape)
    precision = _MATCH_PRECISIONS[match_precision]
    device = noisy.device
    L = _abi.lib()
    if stream is None:
        stream = torch.cuda.current_stream(device)
    sptr = int(stream.cuda_stream)
    params = {}
    schedules = {}
    need = 0
    for stage in ("ht", "wiener"):
        p = plan.stage_params(profile, shape, stage, resolved.blockmatch_distance,
                              resolved.variance_k, precision, None if gauss is None else gauss[stage],
                              null_table_device(profile, resolved, device))
        block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
        counts = tuple(s - b + 1 for s, b in zip(shape, block))
        sched = plan.reference_schedule(profile, counts, stage)
        nbytes = ctypes.c_uint64(0)
        if sigma_maps is not None:
            _abi.check(L.bmnd_stage_sigma_workspace_bytes(ctypes.byref(p), len(sched), ctypes.byref(nbytes)))
        else:
            _abi.check(L.bmnd_stage_workspace_bytes(ctypes.byref(p), len(sched), ctypes.byref(nbytes)))
        need = max(need, nbytes.value)
        params[stage] = (p, counts)
        schedules[stage] = sched
    ws = _WORKSPACE.get(device, need)
    ht_out = torch.empty_like(noisy)
    out = torch.empty_like(noisy)
    pilot = None
    for stage, dst in (("ht", ht_out), ("wiener", out)):
        p, counts = params[stage]
        sched = schedules[stage]
        refs = _device_refs(sched, device)
        sel = cnt = acc = None
        if blockmatch_callback is not None:
            n = len(sched)
            sel = torch.empty((n, p.max_stack), dtype=torch.int32, device=device)
            cnt = torch.empty(n, dtype=torch.int32, device=device)
            acc = torch.empty(n, dtype=torch.int32, device=device)
        if sigma_maps is not None:
            smap = torch.empty_like(noisy)
            _abi.check(L.bmnd_stage_sigma(
                ctypes.byref(p), noisy.data_ptr(), None if pilot is None else pilot.data_ptr(),
                refs.data_ptr(), len(sched), dst.data_ptr(), smap.data_ptr(), float(global_sigma),
                None if sel is None else sel.data_ptr(), None if cnt is None else cnt.data_ptr(),
                None if acc is None else acc.data_ptr(), ws.data_ptr(), ws.numel(), sptr))
            sigma_maps[stage] = smap
        else:
            _abi.check(L.bmnd_stage(
                ctypes.byref(p), noisy.data_ptr(), None if pilot is None else pilot.data_ptr(),
                refs.data_ptr(), len(sched), dst.data_ptr(),
                None if sel is None else sel.data_ptr(), None if cnt is None else cnt.data_ptr(),
                None if acc is None else acc.data_ptr(), ws.data_ptr(), ws.numel(), sptr))
        if blockmatch_callback is not None:
            blockmatch_callback(stage, _match_result(sched, counts, sel.cpu().numpy(),
                                                     cnt.cpu().numpy(), acc.cpu().numpy()))
        if stage_callback is not None:
            stage_callback(stage, dst.cpu().numpy().copy())
        pilot = dst
    return out


def estimate_poisson_global_sigma(volume, eps: float = 1e-10) -> float:
    """Global noise level reported with the sigma maps, as the reference
    computes it (src/bmnd/sigmaestimation.py:48-93): sqrt of the mean of the
    positive values (10%-trimmed when fewer than 10% are positive), with IQR
    and MAD fallbacks."""
    vol = np.asarray(volume, dtype=np.float32)
    finite = np.isfinite(vol)
    nonneg = np.maximum(vol[finite], 0.0) if np.any(finite) else np.array([0.0], dtype=np.float32)
    positive = nonneg[nonneg > 0.0]
    if positive.size > 0:
        frac = positive.size / max(nonneg.size, 1)
        if frac < 0.1 and positive.size >= 3:
            sv = np.sort(positive, axis=None)
            trim = max(int(0.1 * sv.size), 1)
            mean_val = float(np.mean(sv[trim:-trim] if sv.size - 2 * trim > 0 else sv, dtype=np.float32))
        else:
            mean_val = float(np.mean(positive, dtype=np.float32))
    else:
        mean_val = float(np.mean(nonneg, dtype=np.float32))
    g = float(np.sqrt(max(mean_val, eps)))
    if g <= 0.0 and positive.size > 0:
        q25, q75 = np.percentile(positive, [25.0, 75.0])
        if float(q75 - q25) > 0.0:
            g = float(np.sqrt(max(float(q75 - q25) / 1.349, eps)))
    if g <= 0.0 and positive.size > 0:
        med = float(np.median(positive))
        mad = float(np.median(np.abs(positive - med)))
        if mad > 0.0:
            g = float(np.sqrt(max(mad / 0.6745, eps)))
    if g <= 0.0:
        g = float(np.sqrt(eps))
    if not np.isfinite(g) or g < 0.0:
        return 0.0
    return g


def stage_device(noisy, profile, stage: str, pilot=None, *, resolved=None, match_precision: str = "exact",
                 stream=None, gauss: dict | None = None, fast_transforms: bool = False):
    """One filtering stage on a float32 CUDA tensor: "ht" on ``noisy``, or
    "wiener" on ``noisy`` with ``pilot`` as the stage-1 estimate.  Returns the
    stage estimate as a new CUDA tensor.  ``fast_transforms`` selects the Haar
    group axis by its sum pyramid (the fast path's choice)."""
    torch = _torch()
    shape = tuple(int(s) for s in noisy.shape)
    if resolved is None:
        resolved = resolve_profile(profile, shape)
    if stage not in ("ht", "wiener"):
        raise ValueError(f"stage must be 'ht' or 'wiener', got {stage!r}")
    if (stage == "wiener") != (pilot is not None):
        raise ValueError("the Wiener stage needs a pilot and the hard-thresholding stage takes none")
    prep = stage_prepare(noisy, profile, stage, resolved=resolved, match_precision=match_precision, gauss=gauss,
                         fast_transforms=fast_transforms)
    return stage_launch(prep, noisy, pilot, stream=stream)


def stage_prepare(noisy, profile, stage: str, *, resolved=None, match_precision: str = "exact",
                  gauss: dict | None = None, fast_transforms: bool = False) -> dict:
    """The host-side part of :func:`stage_device` (stage parameters, reference
    schedule, workspace, output tensor), so that a caller can do it while the
    device is still busy with earlier work; :func:`stage_launch` runs it."""
    torch = _torch()
    shape = tuple(int(s) for s in noisy.shape)
    if resolved is None:
        resolved = resolve_profile(profile, shape)
    if stage not in ("ht", "wiener"):
        raise ValueError(f"stage must be 'ht' or 'wiener', got {stage!r}")
    precision = _MATCH_PRECISIONS[match_precision]
    device = noisy.device
    L = _abi.lib()
    p = plan.stage_params(profile, shape, stage, resolved.blockmatch_distance, resolved.variance_k, precision,
                          None if gauss is None else gauss[stage], null_table_device(profile, resolved, device),
                          fast_transforms)
    block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    sched = plan.reference_schedule(profile, counts, stage)
    nbytes = ctypes.c_uint64(0)
    _abi.check(L.bmnd_stage_workspace_bytes(ctypes.byref(p), len(sched), ctypes.byref(nbytes)))
    ws = _WORKSPACE.get(device, nbytes.value)
    return dict(stage=stage, params=p, n_refs=len(sched), refs=_device_refs(sched, device), ws=ws,
                out=torch.empty_like(noisy), shape=shape)


def stage_launch(prep: dict, noisy, pilot=None, stream=None):
    """Launch a stage prepared by :func:`stage_prepare`; returns its output tensor."""
    torch = _torch()
    if (prep["stage"] == "wiener") != (pilot is not None):
        raise ValueError("the Wiener stage needs a pilot and the hard-thresholding stage takes none")
    if tuple(int(s) for s in noisy.shape) != prep["shape"]:
        raise ValueError("the volume's shape differs from the prepared stage's")
    if stream is None:
        stream = torch.cuda.current_stream(noisy.device)
    out, ws, refs = prep["out"], prep["ws"], prep["refs"]
    _abi.check(_abi.lib().bmnd_stage(
        ctypes.byref(prep["params"]), noisy.data_ptr(), None if pilot is None else pilot.data_ptr(),
        refs.data_ptr(), prep["n_refs"], out.data_ptr(), None, None, None, ws.data_ptr(), ws.numel(),
        int(stream.cuda_stream)))
    return out


def group_probe(params, noisy, sel, count, pilot=None, stream=None) -> dict:
    """Filter explicit groups on the device and return their intermediate
    arrays (``bmnd_group_probe``): for every group i of ``count[i]`` members
    ``sel[i, :count[i]]`` (patch-grid lins), "coef" (forward transform of the
    observation group), "sigma" (noise std), "atten" (hard-threshold mask or
    Wiener gain) and "filt" (inverse of the shrunk coefficients), each
    n_groups x max_stack x P, and "weights" (n_groups x max_stack), as NumPy
    float32 arrays.  ``params`` is a filled ``StageParams``; ``noisy`` (and
    ``pilot`` for the Wiener filter) are float32 CUDA tensors."""
    torch = _torch()
    L = _abi.lib()
    device = noisy.device
    if stream is None:
        stream = torch.cuda.current_stream(device)
    sel_t = torch.from_numpy(np.ascontiguousarray(sel, dtype=np.int32)).to(device)
    cnt_t = torch.from_numpy(np.ascontiguousarray(count, dtype=np.int32)).to(device)
    n = int(cnt_t.numel())
    P = int(np.prod([params.block[a] for a in range(params.ndim)]))
    nb = ctypes.c_uint64(0)
    _abi.check(L.bmnd_group_probe_workspace_bytes(ctypes.byref(params), ctypes.byref(nb)))
    ws = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device=device)
    out = {k: torch.zeros((n, params.max_stack, P), dtype=torch.float32, device=device)
           for k in ("coef", "sigma", "atten", "filt")}
    out["weights"] = torch.zeros((n, params.max_stack), dtype=torch.float32, device=device)
    _abi.check(L.bmnd_group_probe(
        ctypes.byref(params), noisy.data_ptr(), None if pilot is None else pilot.data_ptr(), sel_t.data_ptr(),
        cnt_t.data_ptr(), n, out["coef"].data_ptr(), out["sigma"].data_ptr(), out["atten"].data_ptr(),
        out["weights"].data_ptr(), out["filt"].data_ptr(), ws.data_ptr(), ws.numel(), int(stream.cuda_stream)))
    return {k: v.cpu().numpy() for k, v in out.items()}


def bmnd(
    volume,
    profile,
    sigma: float | None = None,
    sigma_psd=None,
    return_sigma_map: bool = False,
    stage_callback: Callable[[str, np.ndarray], None] | None = None,
    blockmatch_callback: Callable[[str, BlockMatchResult], None] | None = None,
    max_cache_bytes=CacheMode.AUTO,
    *,
    match_precision: str | None = None,
    pilot: str = "plain",
    pilot_weights: str | None = None,
):
    """Denoise ``volume`` with ``profile`` (drop-in for the reference ``bmnd``).

    ``volume`` may be a NumPy array (the result is a NumPy float32 array of
    the same shape) or a CUDA tensor (the result stays on that device).

    Keyword-only additions, none of which the reference has:

    * ``pilot`` -- "plain" (default) runs the reference's two stages.
      "learned" replaces the hard-thresholding stage by the learned pilot (a
      BF16 residual convolution net on the tensor cores) with its per-tile
      Poisson-deviance fallback to the plain stage 1, then runs the Wiener
      stage with the fast path's settings (``pilot.FAST_STAGE2``: reference
      step 4 and the approximate Poisson sigma in 3-D; subsampled screening
      matching).  Direct-Poisson 2-D and 3-D profiles only; the sigma maps and
      the block-matching callback are not available on it, and
      ``stage_callback`` receives the pilot as the "ht" estimate.
    * ``pilot_weights`` -- the net's ``.npz`` file; default: the weights
      shipped for the volume's dimensionality (``bmnd_gb300/weights``).
    * ``match_precision`` -- "exact" (the default of the plain pilot): float32
      per-term distances for every candidate; "fast": screening plus exact
      rescoring near the selection boundary (same match sets); "approx":
      selection by the screening distances, the selected candidates rescored
      with the ratio form of the deviance (within 4e-6 per unit of r + c of the
      float32 terms; the match sets may differ where the orders disagree); "subsampled" (the default of the learned pilot's Wiener
      stage): "approx" after a prescreen on the patch's even sub-lattice.
    """
    if sigma is not None and sigma_psd is not None:
        raise ValueError("sigma and sigma_psd are mutually exclusive.")
    if sigma is not None:
        _validate_sigma(sigma)
    _validate_max_cache_bytes(max_cache_bytes)
    if pilot not in ("plain", "learned"):
        raise ValueError(f"pilot must be 'plain' or 'learned', got {pilot!r}.")
    if match_precision is not None and match_precision not in _MATCH_PRECISIONS:
        raise ValueError(
            f"match_precision must be 'exact', 'fast', 'approx' or 'subsampled', got {match_precision!r}.")
    learned = pilot == "learned"

    torch_input = type(volume).__module__.startswith("torch")
    shape = tuple(int(s) for s in volume.shape)
    resolved = resolve_profile(profile, shape)
    uploaded = None  # NumPy float32 input already on the device
    if resolved.is_poisson and sigma_psd is not None:
        raise ValueError(
            "sigma_psd is only supported for stationary additive noise; "
            "direct Poisson mode uses a variance volume instead."
        )
    if torch_input:
        torch = _torch()
        dev_vol = volume.detach()
        if not bool(torch.isfinite(dev_vol).all()):
            raise ValueError("volume must contain only finite values.")
        dev_vol = dev_vol.to(torch.float32)
        if not bool(torch.isfinite(dev_vol).all()):
            raise ValueError("volume values must be representable as finite float32 values.")
        if resolved.is_poisson and bool((dev_vol < 0).any()):
            raise ValueError("Direct Poisson input must contain only non-negative values.")
        all_zero = not bool((dev_vol != 0).any())
    else:
        arr = np.asarray(volume)
        if arr.dtype == np.float32 and arr.size:
            # one min and one max pass: NaN propagates through both, so both are
            # finite exactly when every value is (the same checks, in the same order).
            # With a GPU the volume is uploaded first and both are taken there.
            if _cuda_ready():
                uploaded = _STAGING.upload(np.ascontiguousarray(arr))
                mm = _torch().aminmax(uploaded.view(-1))
                lo, hi = (float(v) for v in _torch().stack([mm.min, mm.max]).cpu())
            else:
                lo, hi = float(np.min(arr)), float(np.max(arr))
            if not (np.isfinite(lo) and np.isfinite(hi)):
                raise ValueError("volume must contain only finite values.")
            vol = arr
            if resolved.is_poisson and lo < 0.0:
                raise ValueError("Direct Poisson input must contain only non-negative values.")
            all_zero = lo == 0.0 and hi == 0.0
        else:
            if not np.all(np.isfinite(arr)):
                raise ValueError("volume must contain only finite values.")
            with np.errstate(over="ignore", invalid="ignore"):
                vol = arr.astype(np.float32, copy=False)
            if not np.all(np.isfinite(vol)):
                raise ValueError("volume values must be representable as finite float32 values.")
            if resolved.is_poisson and np.any(vol < 0.0):
                raise ValueError("Direct Poisson input must contain only non-negative values.")
            all_zero = not np.any(vol != 0.0)

    if sigma_psd is not None:
        gaussian.validate_sigma_psd(shape, sigma_psd)

    if all_zero:
        zero = volume if torch_input else vol
        if stage_callback is not None:
            copy = (lambda z: z.cpu().numpy().copy()) if torch_input else (lambda z: z.copy())
            stage_callback("ht", copy(zero))
            stage_callback("wiener", copy(zero))
        if return_sigma_map:
            smap = np.zeros(shape, dtype=np.float32)
            return zero, {"ht": smap, "wiener": smap}
        return zero

    if resolved.is_poisson:
        plan.check_poisson_options(profile, resolved.variance_k)
    else:
        plan.check_gaussian_options(profile, resolved.variance_k)
    if learned:
        if not resolved.is_poisson:
            raise plan.unsupported("the learned pilot is trained for direct-Poisson profiles only")
        if len(shape) not in (2, 3):
            raise plan.unsupported("the learned pilot exists for 2-D and 3-D volumes only")
        if return_sigma_map or blockmatch_callback is not None:
            raise plan.unsupported("return_sigma_map and blockmatch_callback need pilot='plain'")

    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("bmnd_gb300 needs a CUDA device; no CPU fallback exists")
    if torch_input:
        dev = dev_vol.contiguous()
        if not dev.is_cuda:
            dev = dev.cuda()
    elif uploaded is not None:
        dev = uploaded
    else:
        dev = _STAGING.upload(np.ascontiguousarray(vol))
    # the host array of the result, made ready while the device computes
    result_host = None if torch_input else _STAGING.result_buffer(shape)
    maps = None
    global_sigma = 0.0
    gauss = None
    if not resolved.is_poisson:
        host_vol = None
        if sigma is None and sigma_psd is None:
            host_vol = dev.cpu().numpy() if torch_input else vol
        model = gaussian.build_model(shape, profile.nf, sigma=sigma, sigma_psd=sigma_psd, volume=host_vol)
        gauss = gaussian_tables(model, profile, shape, resolved, dev.device)
        if return_sigma_map:
            maps = {}
            global_sigma = model.global_sigma
    elif return_sigma_map:
        maps = {}
        # on the stage-1 variance volume max(scale * max(x, 0), floor) (variance.py:581-592)
        host_vol = dev.cpu().numpy() if torch_input else vol
        floor = float(profile.poisson_variance_floor)
        vvol = np.maximum(np.float32(profile.poisson_count_scale) * np.maximum(host_vol, np.float32(0.0)),
                          np.float32(floor)).astype(np.float32)
        global_sigma = estimate_poisson_global_sigma(vvol, eps=max(floor, 1e-10))
    if learned:
        from . import pilot as pilot_mod

        net = _learned_net(len(shape), pilot_weights, dev.device)
        details = {} if stage_callback is not None else None
        out = pilot_mod.bmnd_fast(dev, profile, net, details=details,
                                  match_precision=match_precision or pilot_mod.FAST_MATCH_PRECISION)
        if stage_callback is not None:
            stage_callback("ht", details["pilot"].cpu().numpy().copy())
            stage_callback("wiener", out.cpu().numpy().copy())
    else:
        out = bmnd_device(dev, profile, resolved=resolved, match_precision=match_precision or "exact",
                          stage_callback=stage_callback, blockmatch_callback=blockmatch_callback,
                          sigma_maps=maps, global_sigma=global_sigma, gauss=gauss)
    if torch_input:
        res = out if volume.is_cuda else out.cpu()
        if maps is None:
            return res
        conv = (lambda t: t) if volume.is_cuda else (lambda t: t.cpu())
        return res, {"global": global_sigma, "ht": conv(maps["ht"]), "wiener": conv(maps["wiener"])}
    if maps is None:
        return _host_result(out, result_host)
    return _host_result(out, result_host), {"global": global_sigma, "ht": maps["ht"].cpu().numpy(),
                               "wiener": maps["wiener"].cpu().numpy()}
