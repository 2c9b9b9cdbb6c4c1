"""Profile dataclasses of the BMND API.

Field names, types and defaults are those of the reference profiles
(src/bmnd/profiles.py:18-405): a profile written for the reference
configures this implementation the same way.  Only the fields that the GPU
path reads are documented here; see the reference for the full semantics.
"""

from __future__ import annotations

from dataclasses import dataclass, field

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
)
from .transforms import Transform, TransformMode, TransformType

__all__ = ["BMNDProfile", "BM2DProfile", "BM3DProfile", "BM4DProfile", "BM5DProfile"]


def _group_haar(spatial: TransformType):
    return lambda: [
        Transform(TransformType.HAAR, TransformMode.GROUP),
        Transform(spatial, TransformMode.SPATIAL),
    ]


@dataclass
class BMNDProfile:
    """Base profile (defaults of src/bmnd/profiles.py:18-174)."""

    noise_model: NoiseModel = NoiseModel.GAUSSIAN
    reference_schedule_mode: ReferenceScheduleMode = ReferenceScheduleMode.GENERATED
    reference_shift_density: float = 2.0
    reference_schedule_density: int = 2
    poisson_variance_source_wiener: PoissonVarianceSource = PoissonVarianceSource.PILOT
    poisson_variance_floor: float = 1e-10
    poisson_count_scale: float = 1.0
    poisson_ht_match_policy: PoissonHTMatchPolicy = PoissonHTMatchPolicy.FIXED
    poisson_wiener_match_source: PoissonVarianceSource = PoissonVarianceSource.PILOT
    poisson_ht_match_structure_beta: float = 0.1
    poisson_ht_match_intensity_power: float = 1.0
    poisson_ht_match_moment_max_count: int = 512
    poisson_wiener_gain_mode: PoissonWienerGainMode = PoissonWienerGainMode.VARIANCE_SCALED
    poisson_group_mass_conservation: PoissonGroupMassConservation = (
        PoissonGroupMassConservation.NONE
    )
    nf: tuple[int, ...] | int | None = field(default_factory=tuple)
    k: int = 4
    ht_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    ht_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    ht_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    wiener_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    wiener_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    wiener_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    denoise_residual: bool = False
    residual_threshold: float = 3.0
    max_pad_size: int = 0
    gamma: float = 1.0
    blockmatch_distance: BlockMatchDistance = BlockMatchDistance.AUTO
    ht_use_soft_thresholding: bool = False
    ht_block_size: tuple[int, ...] = field(default_factory=tuple)
    ht_step: tuple[int, ...] = field(default_factory=tuple)
    ht_search_window: tuple[int, ...] = field(default_factory=tuple)
    ht_max_stack_size: int = field(default_factory=int)
    ht_min_stack_size: int = 2
    ht_match_threshold: float = 2.9527
    ht_lambda_threshold: float = 1.0
    ht_kaiser_beta: float = 2.0
    wiener_block_size: tuple[int, ...] = field(default_factory=tuple)
    wiener_step: tuple[int, ...] = field(default_factory=tuple)
    wiener_search_window: tuple[int, ...] = field(default_factory=tuple)
    wiener_max_stack_size: int = field(default_factory=int)
    wiener_min_stack_size: int = 2
    wiener_match_threshold: float = 0.7689
    wiener_variance_scale: float = 1.0
    wiener_kaiser_beta: float = 2.0
    ht_transform: Transform | list[Transform] = field(
        default_factory=lambda: Transform(TransformType.BIOR15, TransformMode.ND)
    )
    wiener_transform: Transform | list[Transform] = field(
        default_factory=lambda: Transform(TransformType.DCT, TransformMode.ND)
    )
    sharpen_alpha: float = 1.0
    sharpen_alpha_3d: float = 1.0
    ref_batch_size: int = 64


@dataclass
class BM2DProfile(BMNDProfile):
    """One-dimensional signals (src/bmnd/profiles.py:177-222)."""

    noise_model: NoiseModel = NoiseModel.GAUSSIAN
    gamma: float = 3.0
    nf: tuple[int] | int | None = (32,)
    k: int = 4
    ht_use_soft_thresholding: bool = False
    ht_block_size: tuple[int] = (64,)
    ht_step: tuple[int] = (16,)
    ht_search_window: tuple[int] = (128,)
    ht_max_stack_size: int = 16
    ht_min_stack_size: int = 2
    ht_match_threshold: float = 2.9527
    ht_lambda_threshold: float = 3.0
    ht_kaiser_beta: float = 2.0
    wiener_block_size: tuple[int] = (64,)
    wiener_step: tuple[int] = (16,)
    wiener_search_window: tuple[int] = (128,)
    wiener_max_stack_size: int = 32
    wiener_min_stack_size: int = 2
    wiener_match_threshold: float = 0.3937
    wiener_variance_scale: float = 0.4
    wiener_kaiser_beta: float = 2.0
    ht_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.BIOR15))
    wiener_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.DCT))


@dataclass
class BM3DProfile(BMNDProfile):
    """2-D images with the official BM3D parameter values (profiles.py:225-288)."""

    noise_model: NoiseModel = NoiseModel.GAUSSIAN
    gamma: float = 3.0
    nf: tuple[int, int] | int | None = (32, 32)
    k: int = 4
    ht_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    ht_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    ht_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    wiener_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    wiener_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    wiener_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    ht_use_soft_thresholding: bool = False
    ht_block_size: tuple[int, int] = (8, 8)
    ht_step: tuple[int, int] = (3, 3)
    ht_search_window: tuple[int, int] = (19, 19)
    ht_max_stack_size: int = 16
    ht_min_stack_size: int = 2
    ht_match_threshold: float = 2.9527
    ht_lambda_threshold: float = 3.0
    ht_kaiser_beta: float = 2.0
    wiener_block_size: tuple[int, int] = (8, 8)
    wiener_step: tuple[int, int] = (3, 3)
    wiener_search_window: tuple[int, int] = (19, 19)
    wiener_max_stack_size: int = 32
    wiener_min_stack_size: int = 2
    wiener_match_threshold: float = 0.3937
    wiener_variance_scale: float = 0.4
    wiener_kaiser_beta: float = 2.0
    ht_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.BIOR15))
    wiener_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.DCT))
    sharpen_alpha = 1.0
    sharpen_alpha_3d = 1.0
    ref_batch_size: int = 64


@dataclass
class BM4DProfile(BMNDProfile):
    """3-D volumes with the official BM4D parameter values (profiles.py:291-352)."""

    noise_model: NoiseModel = NoiseModel.GAUSSIAN
    gamma: float = 3.0
    nf: tuple[int, int, int] | int | None = (16, 16, 16)
    k: int = 4
    ht_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    ht_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    ht_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    wiener_weight_model: AggregationWeightModel = AggregationWeightModel.VARIANCE
    wiener_weight_domain: AggregationWeightDomain = AggregationWeightDomain.COEFFICIENT
    wiener_weight_scope: AggregationWeightScope = AggregationWeightScope.PATCH
    ht_use_soft_thresholding: bool = False
    ht_block_size: tuple[int, int, int] = (4, 4, 4)
    ht_step: tuple[int, int, int] = (3, 3, 3)
    ht_search_window: tuple[int, int, int] = (7, 7, 7)
    ht_max_stack_size: int = 16
    ht_min_stack_size: int = 2
    ht_match_threshold: float = 2.9527
    ht_lambda_threshold: float = 3.0
    ht_kaiser_beta: float = 2.0
    wiener_block_size: tuple[int, int, int] = (5, 5, 5)
    wiener_step: tuple[int, int, int] = (3, 3, 3)
    wiener_search_window: tuple[int, int, int] = (7, 7, 7)
    wiener_max_stack_size: int = 32
    wiener_min_stack_size: int = 2
    wiener_match_threshold: float = 0.7689
    wiener_variance_scale: float = 0.4
    wiener_kaiser_beta: float = 2.0
    ht_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.BIOR15))
    wiener_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.DCT))
    sharpen_alpha = 1.0
    sharpen_alpha_3d = 1.0
    ref_batch_size: int = 64


@dataclass
class BM5DProfile(BMNDProfile):
    """4-D data (profiles.py:355-405); kept for API completeness (4-D is not on the GPU path)."""

    noise_model: NoiseModel = NoiseModel.GAUSSIAN
    gamma: float = 3.0
    nf: tuple[int, int, int, int] | int | None = (16, 16, 16, 16)
    ht_use_soft_thresholding: bool = False
    ht_block_size: tuple[int, int, int, int] = (4, 4, 4, 4)
    ht_step: tuple[int, int, int, int] = (3, 3, 3, 3)
    ht_search_window: tuple[int, int, int, int] = (3, 3, 7, 7)
    ht_max_stack_size: int = 16
    ht_min_stack_size: int = 2
    ht_match_threshold: float = 2.9527
    ht_lambda_threshold: float = 3.0
    ht_kaiser_beta: float = 2.0
    wiener_block_size: tuple[int, int, int, int] = (4, 4, 4, 4)
    wiener_step: tuple[int, int, int, int] = (3, 3, 3, 3)
    wiener_search_window: tuple[int, int, int, int] = (3, 3, 7, 7)
    wiener_max_stack_size: int = 32
    wiener_min_stack_size: int = 2
    wiener_match_threshold: float = 0.7689
    wiener_variance_scale: float = 1.0
    wiener_kaiser_beta: float = 2.0
    ht_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.BIOR15))
    wiener_transform: Transform | list[Transform] = field(default_factory=_group_haar(TransformType.DCT))
    sharpen_alpha = 1.0
    sharpen_alpha_3d = 1.0
    ref_batch_size: int = 64
