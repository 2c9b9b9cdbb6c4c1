"""Poisson HT match policies: the null moment table behind them.

``null_moment_table`` restates poisson_null_moment_table
(src/bmnd/blockmatching.py:29-83): for a pooled count k = r + c split
binomially (p = 1/2) between reference and candidate, the mean and variance of
one voxel's distance term.  ``reference_finite_count`` thresholds
(blockmatching.py:86-148) and ``candidate_standardized`` distances
(:372-428) are evaluated on the GPU from this table
(``csrc/blockmatch.cu``).
"""

from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

from .enums import BlockMatchDistance


@lru_cache(maxsize=8)
def null_moment_table(distance: BlockMatchDistance, max_count: int = 512) -> np.ndarray:
    """[2, max_count + 1] float64: null means, then null variances."""
    if distance not in (BlockMatchDistance.POISSON_DEVIANCE, BlockMatchDistance.PEARSON,
                        BlockMatchDistance.ANSCOMBE_SSD):
        raise ValueError(
            "Poisson null moments require 'poisson_deviance', 'pearson', "
            f"or 'anscombe_ssd', got {distance!r}."
        )
    if max_count < 1:
        raise ValueError(f"max_count must be positive, got {max_count}.")
    means = np.zeros(max_count + 1, dtype=np.float64)
    variances = np.zeros(max_count + 1, dtype=np.float64)
    if distance is BlockMatchDistance.PEARSON:
        k = np.arange(1, max_count + 1, dtype=np.float64)
        means[1:] = 1.0
        variances[1:] = 2.0 - 2.0 / k
        return np.stack([means, variances])
    for pooled in range(1, max_count + 1):
        e1 = 0.0
        e2 = 0.0
        scale = 2.0 ** (-pooled)
        for r in range(pooled + 1):
            c = pooled - r
            prob = math.comb(pooled, r) * scale
            if distance is BlockMatchDistance.POISSON_DEVIANCE:
                t = 0.0
                if r > 0:
                    t += r * math.log(2.0 * r / pooled)
                if c > 0:
                    t += c * math.log(2.0 * c / pooled)
                t *= 2.0
            else:
                t = 0.5 * (2.0 * math.sqrt(c + 0.375) - 2.0 * math.sqrt(r + 0.375)) ** 2
            e1 += prob * t
            e2 += prob * t * t
        means[pooled] = e1
        variances[pooled] = max(e2 - e1 * e1, 0.0)
    out = np.stack([means, variances])
    out.setflags(write=False)
    return out
