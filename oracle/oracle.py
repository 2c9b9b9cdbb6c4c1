"""ctypes wrappers around the C oracle (test infrastructure only)."""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libbmnd_oracle.so")
LIB64_PATH = os.path.join(HERE, "_ref", "libbmnd_oracle_f64.so")
_lib = None
_lib64 = None

__all__ = [
    "build",
    "load",
    "load_f64",
    "schedule",
    "patch_distance",
    "canonical",
    "blockmatch_patches",
    "blockmatch_volume",
    "blockmatch_volume_poisson_biased",
    "stage",
    "bmnd",
]


def build(force: bool = False) -> str:
    """Compile the oracle (float32 and float64 builds) with its Makefile (gcc only)."""
    src = os.path.getmtime(os.path.join(HERE, "bmnd_oracle.c"))
    stale = any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (LIB_PATH, LIB64_PATH))
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB_PATH


def _bind_stage(L) -> None:
    from bmnd_gb300 import _abi

    i32, i64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    L.oracle_stage.restype = i32
    L.oracle_stage.argtypes = [ctypes.POINTER(_abi.StageParams), vp, vp, vp, i64, vp, vp, vp, vp, i32]
    L.oracle_stage_ex.restype = i32
    L.oracle_stage_ex.argtypes = [ctypes.POINTER(_abi.StageParams), vp, vp, vp, i64, vp, vp, vp, vp, i32, vp,
                                  i32]


def load_f64() -> ctypes.CDLL:
    """The float64-filtering build of the oracle (same matching, float64 transforms,
    noise statistics, shrinkage, weights, aggregation and division)."""
    global _lib64
    if _lib64 is None:
        build()
        L = ctypes.CDLL(LIB64_PATH)
        _bind_stage(L)
        _lib64 = L
    return _lib64


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        from bmnd_gb300 import _abi

        L = ctypes.CDLL(LIB_PATH)
        i32, i64 = ctypes.c_int32, ctypes.c_int64
        vp = ctypes.c_void_p
        L.oracle_schedule.restype = i32
        L.oracle_schedule.argtypes = [i32, vp, vp, vp, ctypes.c_double, i32, vp, vp, vp, i64, vp]
        L.oracle_patch_distance.restype = ctypes.c_float
        L.oracle_patch_distance.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.oracle_patch_distance_f64.restype = ctypes.c_double
        L.oracle_patch_distance_f64.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.oracle_canonical.restype = ctypes.c_float
        L.oracle_canonical.argtypes = [ctypes.c_float]
        L.oracle_blockmatch_patches.restype = i32
        L.oracle_blockmatch_patches.argtypes = [ctypes.POINTER(_abi.MatchParams), vp, i32, vp, i64,
                                                vp, vp, vp, vp, i32, i32]
        L.oracle_blockmatch_volume.restype = i32
        L.oracle_blockmatch_volume.argtypes = [ctypes.POINTER(_abi.MatchParams), vp, vp, vp, vp, i64,
                                               vp, vp, vp, vp, i32, i32]
        L.oracle_blockmatch_volume_biased.restype = i32
        L.oracle_blockmatch_volume_biased.argtypes = [ctypes.POINTER(_abi.MatchParams), vp, vp, vp, vp, i64,
                                                      vp, ctypes.c_float, vp, vp, vp, i32]
        _bind_stage(L)
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def schedule(counts, block, step, shift_density=2.0, schedule_density=2):
    L = load()
    ndim = len(counts)
    c = np.asarray(counts, dtype=np.int32)
    b = np.asarray(block, dtype=np.int32)
    s = np.asarray(step, dtype=np.int32)
    n = ctypes.c_int64(0)
    assert L.oracle_schedule(ndim, _ptr(c), _ptr(b), _ptr(s), shift_density, schedule_density,
                             None, None, None, 0, ctypes.byref(n)) == 0
    a = np.zeros((n.value, ndim), dtype=np.int32)
    sh = np.zeros((n.value, ndim), dtype=np.int32)
    sf = np.zeros((n.value, ndim), dtype=np.int32)
    assert L.oracle_schedule(ndim, _ptr(c), _ptr(b), _ptr(s), shift_density, schedule_density,
                             _ptr(a), _ptr(sh), _ptr(sf), n.value, ctypes.byref(n)) == 0
    return a, sh, sf


def patch_distance(ref, cand, code, count_scale=1.0, f64=False):
    L = load()
    ref = np.ascontiguousarray(ref, dtype=np.float32)
    cand = np.ascontiguousarray(cand, dtype=np.float32)
    fn = L.oracle_patch_distance_f64 if f64 else L.oracle_patch_distance
    return fn(_ptr(ref), _ptr(cand), ref.size, int(code), float(count_scale))


def canonical(d) -> np.ndarray:
    L = load()
    d = np.asarray(d, dtype=np.float32).reshape(-1)
    return np.array([L.oracle_canonical(float(v)) for v in d], dtype=np.float32)


def _match_params(ndim, counts, radius, max_m, min_m, code, stabilize, count_scale, pow2=True):
    from bmnd_gb300 import _abi

    p = _abi.MatchParams()
    p.ndim = ndim
    for a in range(ndim):
        p.counts[a] = int(counts[a])
        p.search_radius[a] = int(radius[a])
    p.max_matches = int(max_m)
    p.min_matches = int(min_m)
    p.prefer_power_of_two = int(pow2)
    p.distance = int(code)
    p.stabilize_ties = int(stabilize)
    p.count_scale = float(count_scale)
    return p


def blockmatch_patches(patches, counts, refs, radius, max_m, min_m, thresholds, code,
                       stabilize=True, count_scale=1.0, pow2=True, f64=False, threads=0):
    L = load()
    patches = np.ascontiguousarray(patches, dtype=np.float32)
    refs = np.ascontiguousarray(refs, dtype=np.int32).reshape(-1, len(counts))
    n = refs.shape[0]
    thr = np.ascontiguousarray(np.broadcast_to(np.asarray(thresholds, dtype=np.float32), (n,)))
    p = _match_params(len(counts), counts, radius, max_m, min_m, code, stabilize, count_scale, pow2)
    sel = np.full((n, max_m), -1, dtype=np.int32)
    cnt = np.zeros(n, dtype=np.int32)
    acc = np.zeros(n, dtype=np.int32)
    assert L.oracle_blockmatch_patches(ctypes.byref(p), _ptr(patches), patches.shape[1], _ptr(refs), n,
                                       _ptr(thr), _ptr(sel), _ptr(cnt), _ptr(acc), int(f64), threads) == 0
    return sel, cnt, acc


def blockmatch_volume(volume, block, refs, radius, max_m, min_m, thresholds, code,
                      stabilize=True, count_scale=1.0, pow2=True, f64=False, threads=0):
    L = load()
    volume = np.ascontiguousarray(volume, dtype=np.float32)
    shape = np.asarray(volume.shape, dtype=np.int32)
    blk = np.asarray(block, dtype=np.int32)
    counts = shape - blk + 1
    refs = np.ascontiguousarray(refs, dtype=np.int32).reshape(-1, volume.ndim)
    n = refs.shape[0]
    thr = np.ascontiguousarray(np.broadcast_to(np.asarray(thresholds, dtype=np.float32), (n,)))
    p = _match_params(volume.ndim, counts, radius, max_m, min_m, code, stabilize, count_scale, pow2)
    sel = np.full((n, max_m), -1, dtype=np.int32)
    cnt = np.zeros(n, dtype=np.int32)
    acc = np.zeros(n, dtype=np.int32)
    assert L.oracle_blockmatch_volume(ctypes.byref(p), _ptr(volume), _ptr(shape), _ptr(blk), _ptr(refs),
                                      n, _ptr(thr), _ptr(sel), _ptr(cnt), _ptr(acc), int(f64), threads) == 0
    return sel, cnt, acc


def blockmatch_volume_poisson_biased(volume, block, refs, radius, max_m, min_m, thresholds, gamma,
                                     count_scale=1.0, pow2=True, threads=0):
    """SSD matching minus gamma times the Poisson pooled-count noise bias
    (blockmatching.py:1140-1145, :432-443)."""
    L = load()
    volume = np.ascontiguousarray(volume, dtype=np.float32)
    shape = np.asarray(volume.shape, dtype=np.int32)
    blk = np.asarray(block, dtype=np.int32)
    counts = shape - blk + 1
    refs = np.ascontiguousarray(refs, dtype=np.int32).reshape(-1, volume.ndim)
    n = refs.shape[0]
    thr = np.ascontiguousarray(np.broadcast_to(np.asarray(thresholds, dtype=np.float32), (n,)))
    p = _match_params(volume.ndim, counts, radius, max_m, min_m, 0, False, count_scale, pow2)
    sel = np.full((n, max_m), -1, dtype=np.int32)
    cnt = np.zeros(n, dtype=np.int32)
    acc = np.zeros(n, dtype=np.int32)
    assert L.oracle_blockmatch_volume_biased(ctypes.byref(p), _ptr(volume), _ptr(shape), _ptr(blk), _ptr(refs),
                                             n, _ptr(thr), float(np.float32(gamma)), _ptr(sel), _ptr(cnt),
                                             _ptr(acc), threads) == 0
    return sel, cnt, acc


def stage(params, noisy, pilot, refs, threads=0, sel=None, count=None, f64=False, margins=False):
    """Run one stage; returns (estimate, sel, count, accepted), plus each
    group's hard-threshold margin when ``margins`` is set.

    With ``sel`` and ``count`` given (n x max_stack and n int32, e.g. another
    implementation's match sets) the stage filters those groups instead of
    matching, which isolates the filtering arithmetic; ``accepted`` is then
    None.  ``f64`` runs the float64-filtering build.  A group's margin is the
    smallest relative distance |c - b| / b of a hard-threshold decision from
    its boundary b (poisson.py:30-46), +inf for Wiener groups."""
    L = load_f64() if f64 else load()
    noisy = np.ascontiguousarray(noisy, dtype=np.float32)
    pilot = None if pilot is None else np.ascontiguousarray(pilot, dtype=np.float32)
    refs = np.ascontiguousarray(refs, dtype=np.int32)
    n = refs.shape[0]
    out = np.empty_like(noisy)
    use_sel = sel is not None
    if use_sel:
        sel = np.ascontiguousarray(sel, dtype=np.int32).reshape(n, params.max_stack).copy()
        cnt = np.ascontiguousarray(count, dtype=np.int32).reshape(n).copy()
        acc = None
    else:
        sel = np.full((n, params.max_stack), -1, dtype=np.int32)
        cnt = np.zeros(n, dtype=np.int32)
        acc = np.zeros(n, dtype=np.int32)
    marg = np.empty(n, dtype=np.float64) if margins else None
    assert L.oracle_stage_ex(ctypes.byref(params), _ptr(noisy), _ptr(pilot), _ptr(refs), n, _ptr(out),
                             _ptr(sel), _ptr(cnt), _ptr(acc), int(use_sel), _ptr(marg), threads) == 0
    return (out, sel, cnt, acc, marg) if margins else (out, sel, cnt, acc)


def bmnd(noisy, profile, threads=0, return_details=False):
    """Both stages for a direct-Poisson profile (bmndalgo.py:71-1063 restated)."""
    from bmnd_gb300 import plan
    from bmnd_gb300.validation import resolve_profile

    vol = np.ascontiguousarray(np.asarray(noisy, dtype=np.float32))
    resolved = resolve_profile(profile, tuple(vol.shape))
    if not np.any(vol != 0.0):
        return (vol, {}) if return_details else vol
    details = {}
    pilot = None
    result = None
    for stage_name in ("ht", "wiener"):
        params = plan.stage_params(profile, vol.shape, stage_name, resolved.blockmatch_distance,
                                   resolved.variance_k)
        block = tuple(getattr(profile, f"{stage_name}_block_size"))
        step = tuple(getattr(profile, f"{stage_name}_step"))
        counts = tuple(s - b + 1 for s, b in zip(vol.shape, block))
        refs, _, _ = schedule(counts, block, step, profile.reference_shift_density,
                              profile.reference_schedule_density)
        est, sel, cnt, acc = stage(params, vol, pilot, refs, threads)
        details[stage_name] = dict(estimate=est, sel=sel, count=cnt, accepted=acc, refs=refs)
        pilot = est
        result = est
    return (result, details) if return_details else result
