"""String enums of the BMND profile API.

Same member names and values as the reference (src/bmnd/enums.py:5-67) so
that profiles written for it keep working, and the same ``ValueError`` text
from :func:`coerce_enum` (src/bmnd/enums.py:73-80).
"""

from __future__ import annotations

from enum import Enum, StrEnum
from typing import TypeVar


class NoiseModel(StrEnum):
    GAUSSIAN = "gaussian"
    POISSON = "poisson"


class ReferenceScheduleMode(StrEnum):
    OFFICIAL = "official"
    GENERATED = "generated"
    BALANCED = "balanced"
    SPARSE = "sparse"
    OFF = "off"


class CacheMode(StrEnum):
    AUTO = "auto"


class BlockMatchDistance(StrEnum):
    AUTO = "auto"
    SSD = "ssd"
    POISSON_DEVIANCE = "poisson_deviance"
    PEARSON = "pearson"
    ANSCOMBE_SSD = "anscombe_ssd"


class AggregationWeightModel(StrEnum):
    CLASSIC = "classic"
    VARIANCE = "variance"
    RISK = "risk"


class AggregationWeightDomain(StrEnum):
    COEFFICIENT = "coefficient"
    WINDOWED_SYNTHESIS = "windowed_synthesis"


class AggregationWeightScope(StrEnum):
    GROUP = "group"
    PATCH = "patch"


class PoissonVarianceSource(StrEnum):
    OBSERVATION = "observation"
    PILOT = "pilot"


class PoissonHTMatchPolicy(StrEnum):
    FIXED = "fixed"
    REFERENCE_FINITE_COUNT = "reference_finite_count"
    CANDIDATE_STANDARDIZED = "candidate_standardized"


class PoissonWienerGainMode(StrEnum):
    CLASSIC = "classic"
    NOISE_FLOOR = "noise-floor"
    VARIANCE_SCALED = "variance-scaled"


class PoissonGroupMassConservation(StrEnum):
    NONE = "none"
    HT = "ht"
    WIENER = "wiener"
    BOTH = "both"


E = TypeVar("E", bound=Enum)


def coerce_enum(value: E | str, enum_type: type[E], name: str) -> E:
    """Return ``value`` as a member of ``enum_type`` or raise ``ValueError``."""
    if isinstance(value, enum_type):
        return value
    try:
        return enum_type(value)
    except (TypeError, ValueError) as exc:
        allowed = ", ".join(repr(member.value) for member in enum_type)
        raise ValueError(f"Unknown {name}: {value!r} (expected {allowed}).") from exc
