"""Host-side planning: stage parameters and reference schedules.

Turns a validated profile and a volume shape into the two ``StageParams``
structs of the C ABI (hard thresholding, Wiener) and the GENERATED reference
schedules, the values the reference derives in bmndalgo.py:230-324 and
:648-743 before it starts filtering.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

from . import _abi
from .enums import (
    AggregationWeightDomain,
    AggregationWeightModel,
    AggregationWeightScope,
    BlockMatchDistance,
    PoissonGroupMassConservation,
    PoissonHTMatchPolicy,
    PoissonVarianceSource,
    PoissonWienerGainMode,
    ReferenceScheduleMode,
)
from .transforms import axis_matrices, resolve_axes

_DISTANCE_CODES = {
    BlockMatchDistance.SSD: _abi.DIST_SSD,
    BlockMatchDistance.POISSON_DEVIANCE: _abi.DIST_POISSON_DEVIANCE,
    BlockMatchDistance.PEARSON: _abi.DIST_PEARSON,
    BlockMatchDistance.ANSCOMBE_SSD: _abi.DIST_ANSCOMBE_SSD,
}
_GROUP_CODES = {"haar": _abi.GROUP_HAAR, "dct": _abi.GROUP_DCT, "none": _abi.GROUP_NONE}
EPS = 1e-10


def kaiser_window(block: tuple[int, ...], beta: float) -> np.ndarray:
    """Separable Kaiser window: float64 outer product stored as float32 (utils.py:5-12)."""
    w = np.kaiser(block[0], beta)
    for n in block[1:]:
        w = np.multiply.outer(w, np.kaiser(n, beta))
    return np.asarray(w, dtype=np.float32)


def _spatial_metric_diag(inverse: list[np.ndarray], window: np.ndarray) -> np.ndarray:
    """diag(S^T diag(w^2) S) for the kron S of the inverse spatial matrices (float64)."""
    synth = np.ones((1, 1), dtype=np.float64)
    for m in inverse:
        synth = np.kron(synth, np.asarray(m, dtype=np.float64))
    w2 = np.asarray(window, dtype=np.float64).reshape(-1) ** 2
    metric = synth.T @ (w2[:, None] * synth)
    return np.diag(metric).copy()


def unsupported(reason: str) -> NotImplementedError:
    return NotImplementedError(f"bmnd_gb300: {reason}")


def spatial_forward(profile, ndim: int, stage: str) -> list:
    """Per-axis forward spatial matrices of ``stage`` (None: identity)."""
    block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
    _, spatial = resolve_axes(getattr(profile, f"{stage}_transform"), ndim)
    return [None if kind is None else axis_matrices(kind, block[a])[0] for a, kind in enumerate(spatial)]


def stage_params(profile, shape: tuple[int, ...], stage: str, distance: BlockMatchDistance,
                 variance_k: int, match_precision: int = _abi.MATCH_EXACT, gauss: dict | None = None,
                 null_table=None, fast_transforms: bool = False) -> _abi.StageParams:
    """Fill the ``StageParams`` of ``stage`` ("ht" or "wiener").

    ``gauss`` (stationary Gaussian noise) holds the device tables of the stage:
    ``cov`` (float32 CUDA tensor [lag][coefficient]), ``domain`` (its lag
    domain), ``ssd`` (SSD noise bias over the search offsets, or None) and
    ``gamma``, and ``white_variance`` (the noise variance when the noise is
    white, else None); without it the stage models direct Poisson noise.  ``null_table``
    (float64 CUDA tensor [2, max_count + 1], ``policies.null_moment_table``)
    enables the profile's Poisson HT match policy.  ``fast_transforms`` computes
    the Haar group axis by its sum pyramid (same transform, different rounding)."""
    ndim = len(shape)
    if ndim < 1 or ndim > _abi.MAX_DIMS:
        raise unsupported(f"{ndim}-D volumes are not supported (1 to {_abi.MAX_DIMS} dimensions)")
    block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
    radius = tuple(int(r) for r in getattr(profile, f"{stage}_search_window"))
    max_stack = int(getattr(profile, f"{stage}_max_stack_size"))
    min_stack = int(getattr(profile, f"{stage}_min_stack_size"))
    if any(b > _abi.MAX_EDGE for b in block):
        raise unsupported(f"patch edges above {_abi.MAX_EDGE} are not supported, got {block}")
    if max_stack > _abi.MAX_STACK:
        raise unsupported(f"stack sizes above {_abi.MAX_STACK} are not supported, got {max_stack}")
    model = getattr(profile, f"{stage}_weight_model")
    domain = getattr(profile, f"{stage}_weight_domain")
    scope = getattr(profile, f"{stage}_weight_scope")
    exact_risk = _check_stage_weights(stage, model, domain, scope, variance_k, int(np.prod(block)))

    group_kind, spatial = resolve_axes(getattr(profile, f"{stage}_transform"), ndim)
    p = _abi.StageParams()
    p.ndim = ndim
    for a in range(ndim):
        p.shape[a] = int(shape[a])
        p.block[a] = block[a]
        p.search_radius[a] = radius[a]
    p.max_stack = max_stack
    p.min_stack = min_stack
    p.distance = _DISTANCE_CODES[distance]
    p.stabilize_ties = 0 if gauss is not None else 1
    p.match_precision = match_precision
    p.filter = _abi.FILTER_HARD_THRESHOLD if stage == "ht" else _abi.FILTER_WIENER
    p.group_transform = _GROUP_CODES[group_kind]
    p.variance_k = int(variance_k)
    p.weight_model = {AggregationWeightModel.VARIANCE: _abi.WEIGHT_VARIANCE,
                      AggregationWeightModel.CLASSIC: _abi.WEIGHT_CLASSIC,
                      AggregationWeightModel.RISK: _abi.WEIGHT_RISK}[model]
    p.weight_group_scope = int(scope is AggregationWeightScope.GROUP)
    p.fast_group_transform = int(bool(fast_transforms))
    p.windowed_synthesis = int(domain is AggregationWeightDomain.WINDOWED_SYNTHESIS)
    # exact risk weights under Gaussian noise only when the noise is white
    # (variance.py:1459-1470); otherwise the reference weighs by the diagonal
    if exact_risk and (gauss is None or gauss.get("white_variance") is not None):
        p.exact_risk_weights = 1
        if gauss is not None:
            p.exact_source_variance = float(np.float32(gauss["white_variance"]))
    p.match_threshold = float(np.float32(getattr(profile, f"{stage}_match_threshold")))
    p.ht_lambda = float(profile.ht_lambda_threshold)
    p.wiener_scale = float(profile.wiener_variance_scale)
    p.eps = EPS
    p.ssd_threshold = float(getattr(profile, f"{stage}_match_threshold"))
    p.soft_threshold = int(stage == "ht" and bool(profile.ht_use_soft_thresholding))
    if gauss is None:
        p.noise_model = _abi.NOISE_POISSON
        p.count_scale = float(profile.poisson_count_scale)
        if stage == "ht" and distance is BlockMatchDistance.SSD and float(profile.gamma) != 0.0:
            # Poisson SSD noise bias, hard thresholding only (bmndalgo.py:292-294,
            # blockmatching.py:244-262, :1140-1145); gamma reaches the kernel as float32
            p.ssd_poisson_bias = 1
            p.ssd_gamma = float(np.float32(profile.gamma))
        p.variance_floor = float(profile.poisson_variance_floor)
        gain = profile.poisson_wiener_gain_mode
        p.wiener_gain_mode = {PoissonWienerGainMode.VARIANCE_SCALED: _abi.GAIN_VARIANCE_SCALED,
                              PoissonWienerGainMode.CLASSIC: _abi.GAIN_CLASSIC,
                              PoissonWienerGainMode.NOISE_FLOOR: _abi.GAIN_NOISE_FLOOR}[gain]
        obs = PoissonVarianceSource.OBSERVATION
        p.wiener_variance_source = _abi.SOURCE_OBSERVATION if profile.poisson_variance_source_wiener is obs \
            else _abi.SOURCE_PILOT
        p.wiener_match_source = _abi.SOURCE_OBSERVATION if profile.poisson_wiener_match_source is obs \
            else _abi.SOURCE_PILOT
        policy = profile.poisson_ht_match_policy
        if stage == "ht" and policy is not PoissonHTMatchPolicy.FIXED:
            if null_table is None:
                raise ValueError("the Poisson HT match policy needs the null moment table")
            p.match_policy = (_abi.POLICY_REFERENCE_FINITE_COUNT
                              if policy is PoissonHTMatchPolicy.REFERENCE_FINITE_COUNT
                              else _abi.POLICY_CANDIDATE_STANDARDIZED)
            p.null_max_count = int(profile.poisson_ht_match_moment_max_count)
            p.null_moments = null_table.data_ptr()
            p.policy_beta = float(profile.poisson_ht_match_structure_beta)
            p.policy_power = float(profile.poisson_ht_match_intensity_power)
        mass = profile.poisson_group_mass_conservation
        p.mass_conserve = int(mass is PoissonGroupMassConservation.BOTH
                              or (mass is PoissonGroupMassConservation.HT and stage == "ht")
                              or (mass is PoissonGroupMassConservation.WIENER and stage == "wiener"))
    else:
        p.noise_model = _abi.NOISE_GAUSSIAN
        p.count_scale = 1.0
        p.variance_floor = 0.0
        for a, n in enumerate(gauss["domain"]):
            p.cov_domain[a] = int(n)
        p.cov_maps = gauss["cov"].data_ptr()
        if gauss.get("ssd") is not None:
            p.match_noise_ssd = gauss["ssd"].data_ptr()
            p.ssd_gamma = float(gauss["gamma"])
    inverse = []
    for a in range(ndim):
        kind = spatial[a]
        if kind is None:
            fwd = np.eye(block[a], dtype=np.float32)
            inv = fwd
        else:
            fwd, inv = axis_matrices(kind, block[a])
        inverse.append(inv)
        flat_f = np.zeros(_abi.MAX_EDGE * _abi.MAX_EDGE, dtype=np.float32)
        flat_i = np.zeros(_abi.MAX_EDGE * _abi.MAX_EDGE, dtype=np.float32)
        flat_f[: block[a] * block[a]] = np.asarray(fwd, dtype=np.float32).reshape(-1)
        flat_i[: block[a] * block[a]] = np.asarray(inv, dtype=np.float32).reshape(-1)
        ctypes.memmove(p.spatial_fwd[a], flat_f.ctypes.data, flat_f.nbytes)
        ctypes.memmove(p.spatial_inv[a], flat_i.ctypes.data, flat_i.nbytes)
    window = kaiser_window(block, float(getattr(profile, f"{stage}_kaiser_beta"))).reshape(-1)
    if window.size > _abi.MAX_PATCH:
        raise unsupported(f"patch volume {window.size} exceeds {_abi.MAX_PATCH}")
    wbuf = np.zeros(_abi.MAX_PATCH, dtype=np.float32)
    wbuf[: window.size] = window
    ctypes.memmove(p.window, wbuf.ctypes.data, wbuf.nbytes)
    if p.windowed_synthesis:
        diag = np.zeros(_abi.MAX_PATCH, dtype=np.float64)
        diag[: window.size] = _spatial_metric_diag(inverse, window)
        ctypes.memmove(p.spatial_metric_diag, diag.ctypes.data, diag.nbytes)
    return p


def _check_stage_weights(stage, model, domain, scope, variance_k, patch_volume: int) -> bool:
    """Whether the stage weights its groups by their exact risk: the
    covariance-aware exact group weighting (bmndalgo.py:363-370, :752-758)."""
    if model is AggregationWeightModel.RISK and stage != "wiener":
        raise unsupported("risk aggregation weights apply to the Wiener stage only")
    exact = (model in (AggregationWeightModel.VARIANCE, AggregationWeightModel.RISK)
             and domain is AggregationWeightDomain.WINDOWED_SYNTHESIS
             and scope is AggregationWeightScope.GROUP and int(variance_k) > 0)
    if exact and patch_volume > 128:
        raise unsupported(f"the covariance-aware exact group weighting needs patches of at most 128 voxels, "
                          f"got {patch_volume}")
    return exact


def check_weight_options(profile, variance_k: int) -> None:
    """Reject the aggregation-weight options that are not on the GPU path."""
    for stage in ("ht", "wiener"):
        _check_stage_weights(stage, getattr(profile, f"{stage}_weight_model"),
                             getattr(profile, f"{stage}_weight_domain"),
                             getattr(profile, f"{stage}_weight_scope"), variance_k,
                             int(np.prod(getattr(profile, f"{stage}_block_size"))))


def check_gaussian_options(profile, variance_k: int) -> None:
    """Reject the Gaussian options that are not on the GPU path."""
    check_weight_options(profile, variance_k)
    if profile.reference_schedule_mode not in (
        ReferenceScheduleMode.GENERATED,
        ReferenceScheduleMode.OFF,
    ):
        raise unsupported(
            f"reference schedule {profile.reference_schedule_mode.value!r} is not on the GPU path"
        )


def check_poisson_options(profile, variance_k: int) -> None:
    """Reject the non-default Poisson options that are not on the GPU path."""
    check_weight_options(profile, variance_k)
    if profile.reference_schedule_mode not in (
        ReferenceScheduleMode.GENERATED,
        ReferenceScheduleMode.OFF,
    ):
        raise unsupported(
            f"reference schedule {profile.reference_schedule_mode.value!r} is not on the GPU path"
        )


@dataclass(frozen=True)
class Schedule:
    """Reference schedule: per group reference_abs, reference_shifted, shift (n x ndim int32)."""

    reference_abs: np.ndarray
    reference_shifted: np.ndarray
    shift: np.ndarray

    def __len__(self) -> int:
        return int(self.reference_abs.shape[0])


@lru_cache(maxsize=32)
def _generated_schedule(counts, block, step, shift_density, schedule_density) -> Schedule:
    L = _abi.lib()
    ndim = len(counts)
    c = (ctypes.c_int32 * ndim)(*counts)
    b = (ctypes.c_int32 * ndim)(*block)
    s = (ctypes.c_int32 * ndim)(*step)
    n = ctypes.c_int64(0)
    _abi.check(L.bmnd_reference_schedule(ndim, c, b, s, float(shift_density), int(schedule_density),
                                         None, None, None, 0, ctypes.byref(n)))
    abs_ = np.zeros((n.value, ndim), dtype=np.int32)
    shifted = np.zeros((n.value, ndim), dtype=np.int32)
    shift = np.zeros((n.value, ndim), dtype=np.int32)
    i32p = ctypes.POINTER(ctypes.c_int32)
    _abi.check(L.bmnd_reference_schedule(
        ndim, c, b, s, float(shift_density), int(schedule_density),
        abs_.ctypes.data_as(i32p), shifted.ctypes.data_as(i32p), shift.ctypes.data_as(i32p),
        n.value, ctypes.byref(n)))
    for arr in (abs_, shifted, shift):
        arr.setflags(write=False)
    return Schedule(abs_, shifted, shift)


def _off_schedule(counts, step) -> Schedule:
    """Unshifted lattice with the last position forced (shifts.py:486-516)."""
    per_axis = []
    for count, st in zip(counts, step):
        last = max(int(count) - 1, 0)
        starts = list(range(0, last + 1, int(st)))
        if starts[-1] != last:
            starts.append(last)
        per_axis.append(np.asarray(starts, dtype=np.int32))
    grids = np.meshgrid(*per_axis, indexing="ij")
    abs_ = np.stack([g.reshape(-1) for g in grids], axis=1).astype(np.int32)
    return Schedule(abs_, abs_.copy(), np.zeros_like(abs_))


def reference_schedule(profile, counts: tuple[int, ...], stage: str) -> Schedule:
    block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
    step = tuple(int(s) for s in getattr(profile, f"{stage}_step"))
    if profile.reference_schedule_mode is ReferenceScheduleMode.OFF:
        return _off_schedule(counts, step)
    return _generated_schedule(tuple(int(c) for c in counts), block, step,
                               float(profile.reference_shift_density),
                               int(profile.reference_schedule_density))
