"""Profile validation with the reference's rules and messages.

Restates resolve_profile (src/bmnd/profilevalidation.py:33-456): the same
checks in the same order, the same ``ValueError`` texts, and the same in-place
enum coercion of the caller's profile (profilevalidation.py:133-134, :219,
:250-252).  The Gaussian branch resolves the local-variance domain ``nf``
(psd.py:57-98, restated in ``gaussian.resolve_nf``); conventional mode (a
zero ``nf``) sets ``k`` to 0, as the reference does (profilevalidation.py:445-448).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .enums import (
    AggregationWeightDomain,
    AggregationWeightModel,
    AggregationWeightScope,
    BlockMatchDistance,
    NoiseModel,
    PoissonGroupMassConservation,
    PoissonHTMatchPolicy,
    PoissonVarianceSource,
    PoissonWienerGainMode,
    ReferenceScheduleMode,
    coerce_enum,
)
from .gaussian import resolve_nf
from .transforms import Transform, TransformMode, TransformType

_OPERATOR_TYPES = {
    TransformType.STARLET,
    TransformType.ATROUS,
    TransformType.B3SPLINE,
    TransformType.CURVELET,
}


@dataclass(frozen=True)
class ResolvedProfile:
    is_poisson: bool
    effective_nf: tuple[int, ...] | None
    conventional_nf: bool
    blockmatch_distance: BlockMatchDistance
    variance_k: int


def resolve_blockmatch_distance(distance, noise_model) -> BlockMatchDistance:
    """AUTO -> Poisson deviance for Poisson noise, SSD otherwise (blockmatching.py:187-206)."""
    distance = coerce_enum(distance, BlockMatchDistance, "block-matching distance")
    noise_model = coerce_enum(noise_model, NoiseModel, "noise_model")
    if distance is BlockMatchDistance.AUTO:
        return (
            BlockMatchDistance.POISSON_DEVIANCE
            if noise_model is NoiseModel.POISSON
            else BlockMatchDistance.SSD
        )
    return distance


def _finite_nonnegative(name: str, value: object) -> float:
    if isinstance(value, (bool, np.bool_)):
        raise ValueError(f"{name} must be finite and non-negative, got {value!r}.")
    try:
        result = float(value)
    except (TypeError, ValueError) as exc:
        raise ValueError(f"{name} must be finite and non-negative, got {value!r}.") from exc
    if not np.isfinite(result) or result < 0.0:
        raise ValueError(f"{name} must be finite and non-negative, got {value!r}.")
    return result


def _is_int(value: object) -> bool:
    return not isinstance(value, (bool, np.bool_)) and isinstance(value, (int, np.integer))


def _axis_values(name, values, shape, *, minimum, maximum=None) -> None:
    try:
        items = tuple(values)
    except TypeError as exc:
        raise ValueError(
            f"{name} must contain {len(shape)} integer values, got {values!r}."
        ) from exc
    if len(items) != len(shape):
        raise ValueError(
            f"{name} must contain {len(shape)} values for shape {shape}, got {items}."
        )
    if any(isinstance(v, bool) or not isinstance(v, (int, np.integer)) for v in items):
        raise ValueError(f"{name} values must be integers, got {items}.")
    if any(int(v) < minimum for v in items):
        qualifier = "positive" if minimum == 1 else "non-negative"
        raise ValueError(f"{name} values must be {qualifier}, got {items}.")
    if maximum is not None and any(int(v) > maximum[i] for i, v in enumerate(items)):
        raise ValueError(f"{name} values cannot exceed volume shape {maximum}, got {items}.")


def _stack_sizes(stage: str, minimum, maximum) -> None:
    for name, value in ((f"{stage}_min_stack_size", minimum), (f"{stage}_max_stack_size", maximum)):
        if isinstance(value, bool) or not isinstance(value, (int, np.integer)) or int(value) <= 0:
            raise ValueError(f"{name} must be a positive integer, got {value!r}.")
    if int(minimum) > int(maximum):
        raise ValueError(
            f"{stage}_min_stack_size cannot exceed {stage}_max_stack_size, "
            f"got {minimum} > {maximum}."
        )


def _transform_list(name: str, transform) -> list[Transform]:
    if type(transform) is Transform:
        items = [transform]
    elif type(transform) is list:
        items = transform
    else:
        raise ValueError(f"{name} must be a Transform or list of Transform objects.")
    for t in items:
        if type(t) is not Transform:
            raise ValueError(f"{name} must contain only Transform objects.")
        if not isinstance(t.type, TransformType):
            raise ValueError(f"{name} contains an unknown transform type: {t.type!r}.")
        if not isinstance(t.mode, TransformMode):
            raise ValueError(f"{name} contains an unknown transform mode: {t.mode!r}.")
    return items


def resolve_profile(profile, volume_shape: tuple[int, ...]) -> ResolvedProfile:
    """Validate ``profile`` for a volume of ``volume_shape``; coerce its enums in place."""
    noise_model = coerce_enum(profile.noise_model, NoiseModel, "noise_model")
    profile.noise_model = noise_model
    mode = coerce_enum(profile.reference_schedule_mode, ReferenceScheduleMode, "reference_schedule_mode")
    profile.reference_schedule_mode = mode
    if mode in {
        ReferenceScheduleMode.GENERATED,
        ReferenceScheduleMode.BALANCED,
        ReferenceScheduleMode.SPARSE,
    }:
        _finite_nonnegative("reference_shift_density", profile.reference_shift_density)
        density = profile.reference_schedule_density
        if not _is_int(density) or int(density) <= 0:
            raise ValueError(
                f"reference_schedule_density must be a positive integer, got {density!r}."
            )

    for stage in ("ht", "wiener"):
        _axis_values(f"{stage}_block_size", getattr(profile, f"{stage}_block_size"), volume_shape,
                     minimum=1, maximum=volume_shape)
        _axis_values(f"{stage}_step", getattr(profile, f"{stage}_step"), volume_shape, minimum=1)
        _axis_values(f"{stage}_search_window", getattr(profile, f"{stage}_search_window"),
                     volume_shape, minimum=0)
        _stack_sizes(stage, getattr(profile, f"{stage}_min_stack_size"),
                     getattr(profile, f"{stage}_max_stack_size"))
        _transform_list(f"{stage}_transform", getattr(profile, f"{stage}_transform"))
        _finite_nonnegative(f"{stage}_match_threshold", getattr(profile, f"{stage}_match_threshold"))
        _finite_nonnegative(f"{stage}_kaiser_beta", getattr(profile, f"{stage}_kaiser_beta"))

    _finite_nonnegative("ht_lambda_threshold", profile.ht_lambda_threshold)
    _finite_nonnegative("wiener_variance_scale", profile.wiener_variance_scale)
    batch = profile.ref_batch_size
    if not _is_int(batch) or int(batch) <= 0:
        raise ValueError(f"ref_batch_size must be a positive integer, got {batch!r}.")

    configured = coerce_enum(profile.blockmatch_distance, BlockMatchDistance, "blockmatch_distance")
    profile.blockmatch_distance = configured
    distance = resolve_blockmatch_distance(configured, noise_model)
    is_poisson = noise_model is NoiseModel.POISSON

    k = profile.k
    if isinstance(k, bool) or not isinstance(k, (int, np.integer)):
        raise ValueError(f"k must be a non-negative integer, got {k!r}.")
    if int(k) < 0:
        raise ValueError(f"k must be a non-negative integer, got {k!r}.")
    variance_k = int(k)

    for stage in ("ht", "wiener"):
        model_name, domain_name, scope_name = (
            f"{stage}_weight_model",
            f"{stage}_weight_domain",
            f"{stage}_weight_scope",
        )
        model = coerce_enum(getattr(profile, model_name), AggregationWeightModel, model_name)
        domain = coerce_enum(getattr(profile, domain_name), AggregationWeightDomain, domain_name)
        scope = coerce_enum(getattr(profile, scope_name), AggregationWeightScope, scope_name)
        setattr(profile, model_name, model)
        setattr(profile, domain_name, domain)
        setattr(profile, scope_name, scope)
        allowed = {AggregationWeightModel.CLASSIC, AggregationWeightModel.VARIANCE}
        if stage == "wiener":
            allowed.add(AggregationWeightModel.RISK)
        if model not in allowed:
            expected = "', '".join(sorted(allowed))
            raise ValueError(f"Unknown {model_name}: {model!r} (expected '{expected}').")
        configured_t = getattr(profile, f"{stage}_transform")
        items = [configured_t] if type(configured_t) is Transform else configured_t
        all_synthesis = domain is AggregationWeightDomain.WINDOWED_SYNTHESIS
        group_synthesis = scope is AggregationWeightScope.PATCH
        for t in items:
            on_group = t.mode in {TransformMode.ND, TransformMode.GROUP}
            if not all_synthesis and not (group_synthesis and on_group):
                continue
            if t.type in _OPERATOR_TYPES:
                raise ValueError(
                    f"{stage.upper()} {domain}/{scope} weighting requires matrix-based transforms."
                )
            if t.type is TransformType.FFT:
                raise ValueError(
                    f"{stage.upper()} {domain}/{scope} weighting requires real matrix transforms."
                )

    if profile.sharpen_alpha != 1.0 or profile.sharpen_alpha_3d != 1.0:
        raise ValueError("Aggregation weighting requires sharpening exponents of 1.")

    gamma = float(profile.gamma)
    if not np.isfinite(gamma) or gamma < 0.0:
        raise ValueError(f"gamma must be finite and non-negative, got {profile.gamma}.")

    effective_nf = None
    conventional_nf = False
    if is_poisson:
        for name, enum_type in (
            ("poisson_ht_match_policy", PoissonHTMatchPolicy),
            ("poisson_wiener_gain_mode", PoissonWienerGainMode),
            ("poisson_group_mass_conservation", PoissonGroupMassConservation),
        ):
            setattr(profile, name, coerce_enum(getattr(profile, name), enum_type, name))
        profile.poisson_variance_source_wiener = coerce_enum(
            profile.poisson_variance_source_wiener, PoissonVarianceSource,
            "poisson_variance_source_wiener",
        )
        profile.poisson_wiener_match_source = coerce_enum(
            profile.poisson_wiener_match_source, PoissonVarianceSource,
            "poisson_wiener_match_source",
        )
        scale = float(profile.poisson_count_scale)
        if not np.isfinite(scale) or scale <= 0.0:
            raise ValueError(
                "poisson_count_scale must be finite and positive, "
                f"got {profile.poisson_count_scale}."
            )
        _finite_nonnegative("poisson_variance_floor", profile.poisson_variance_floor)
        mass = profile.poisson_group_mass_conservation
        if mass in {PoissonGroupMassConservation.WIENER, PoissonGroupMassConservation.BOTH}:
            if profile.sharpen_alpha != 1.0 or profile.sharpen_alpha_3d != 1.0:
                raise ValueError("Wiener group-mass conservation requires sharpening exponents of 1.")
            wt = profile.wiener_transform
            witems = [wt] if type(wt) is Transform else wt
            if profile.wiener_weight_model in {
                AggregationWeightModel.VARIANCE,
                AggregationWeightModel.RISK,
            } and any(t.type is TransformType.FFT for t in witems):
                raise ValueError(
                    "Mass-projected Poisson Wiener weighting requires real matrix transforms."
                )
        for stage, enabled in (
            ("ht", mass in {PoissonGroupMassConservation.HT, PoissonGroupMassConservation.BOTH}),
            ("wiener", mass in {PoissonGroupMassConservation.WIENER, PoissonGroupMassConservation.BOTH}),
        ):
            if not enabled:
                continue
            st = getattr(profile, f"{stage}_transform")
            sitems = [st] if type(st) is Transform else st
            if any(t.type in _OPERATOR_TYPES for t in sitems):
                raise ValueError(
                    f"{stage.upper()} group-mass conservation requires matrix-based transforms."
                )
            projected = getattr(profile, f"{stage}_weight_model") in {
                AggregationWeightModel.VARIANCE,
                AggregationWeightModel.RISK,
            }
            if projected and any(t.type is TransformType.FFT for t in sitems):
                raise ValueError(
                    f"Mass-projected Poisson {stage.upper()} weighting requires real matrix transforms."
                )
        max_count = profile.poisson_ht_match_moment_max_count
        if not _is_int(max_count) or int(max_count) <= 0:
            raise ValueError(
                "poisson_ht_match_moment_max_count must be a positive integer, "
                f"got {max_count!r}."
            )
        policy = profile.poisson_ht_match_policy
        if policy is not PoissonHTMatchPolicy.FIXED and distance not in {
            BlockMatchDistance.POISSON_DEVIANCE,
            BlockMatchDistance.PEARSON,
            BlockMatchDistance.ANSCOMBE_SSD,
        }:
            raise ValueError(
                f"Poisson HT match policy {policy!r} requires 'poisson_deviance', "
                f"'pearson', or 'anscombe_ssd', got {distance!r}."
            )
        if policy is PoissonHTMatchPolicy.REFERENCE_FINITE_COUNT:
            for name, value, positive in (
                ("poisson_ht_match_structure_beta", float(profile.poisson_ht_match_structure_beta), False),
                ("poisson_ht_match_intensity_power", profile.poisson_ht_match_intensity_power, True),
            ):
                if not np.isfinite(value) or value < 0.0 or (positive and value == 0.0):
                    qualifier = "positive" if positive else "non-negative"
                    raise ValueError(f"{name} must be finite and {qualifier}, got {value}.")
    else:
        effective_nf, conventional_nf = resolve_nf(profile.nf, tuple(int(s) for s in volume_shape))
        if conventional_nf:
            variance_k = 0

    return ResolvedProfile(
        is_poisson=is_poisson,
        effective_nf=effective_nf,
        conventional_nf=conventional_nf,
        blockmatch_distance=distance,
        variance_k=variance_k,
    )
