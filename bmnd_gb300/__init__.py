"""GB300-native (sm_103a) BMND collaborative-filtering path.

Drop-in for the reference package's public API (src/bmnd/__init__.py:1-35):
``bmnd``, the profile dataclasses and the enums.  The work below argument
validation runs in ``libbmnd_gb300.so`` (hand-written CUDA kernels behind the
C ABI in include/bmnd_gb300.h).
"""

from .api import BlockMatchGroup, BlockMatchResult, bmnd, bmnd_device
from .enums import (
    AggregationWeightDomain,
    AggregationWeightModel,
    AggregationWeightScope,
    BlockMatchDistance,
    CacheMode,
    NoiseModel,
    PoissonGroupMassConservation,
    PoissonHTMatchPolicy,
    PoissonVarianceSource,
    PoissonWienerGainMode,
    ReferenceScheduleMode,
)
from .profiles import BM2DProfile, BM3DProfile, BM4DProfile, BM5DProfile, BMNDProfile
from .transforms import Transform, TransformMode, TransformType

__all__ = [
    "AggregationWeightDomain",
    "AggregationWeightModel",
    "AggregationWeightScope",
    "BM2DProfile",
    "BM3DProfile",
    "BM4DProfile",
    "BM5DProfile",
    "BMNDProfile",
    "BlockMatchDistance",
    "BlockMatchGroup",
    "BlockMatchResult",
    "CacheMode",
    "NoiseModel",
    "PoissonGroupMassConservation",
    "PoissonHTMatchPolicy",
    "PoissonVarianceSource",
    "PoissonWienerGainMode",
    "ReferenceScheduleMode",
    "Transform",
    "TransformMode",
    "TransformType",
    "bmnd",
    "bmnd_device",
]
