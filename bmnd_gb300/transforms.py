"""Transform descriptors and the per-axis matrices the GPU path applies.

``TransformType`` / ``TransformMode`` / ``Transform`` keep the reference's
names and values (src/bmnd/transforms.py:73-102) so profiles carry over.

The matrices are built here on the host, in float32, the way the reference
builds them, and handed to the library as per-axis forward/inverse pairs:

* DCT-II, orthonormal (transforms.py:359-386): float64 cosines stored as float32.
* DST-I (transforms.py:494-513) and normalised Hadamard (:556-565).
* bior1.5 for lengths 4 and 8: the tabulated BM3D/BM4D analysis matrices
  (transforms.py:705-806); the synthesis matrix is their inverse, computed
  here in float64 and rounded to float32.  These tables must equal the
  reference's values because the reference filters with exactly them.
* The group axis uses the hierarchical Haar matrix for power-of-two group
  sizes and the DCT-II otherwise (transforms.py:393-440).  The library builds
  those matrices itself for every group size.

Other types (FFT, the pywt-backed wavelets, the operator transforms) are not
available on the GPU path and raise ``NotImplementedError``.
"""

from __future__ import annotations

import enum
from dataclasses import dataclass, field
from typing import Any

import numpy as np


class TransformType(enum.Enum):
    DCT = 0
    FFT = 1
    DST = 2
    HAAR = 3
    HADAMARD = 4
    BIOR15 = 5
    BIOR22 = 6
    BIOR33 = 7
    DB1 = 8
    DB2 = 9
    STARLET = 10
    ATROUS = 11
    B3SPLINE = 12
    CURVELET = 13


class TransformMode(enum.Enum):
    ND = 0
    GROUP = 1
    SPATIAL = 2


@dataclass
class Transform:
    type: TransformType
    mode: TransformMode
    parameters: dict[str, Any] = field(default_factory=dict)


# bior1.5 analysis matrices used by BM3D/BM4D for 4- and 8-point patches.
_BIOR15_4 = (
    (0.5, 0.5, 0.5, 0.5),
    (0.5, 0.5, -0.5, -0.5),
    (0.70710677, -0.70710677, 0.0, 0.0),
    (0.0, 0.0, 0.70710677, -0.70710677),
)
_B8_A = 0.343550200747110
_B8_B = 0.225454819240296
_B8_C = 0.461645582253923
_B8_D = 0.569359398342840
_B8_E = 0.402347308162280
_B8_F = 0.083506045090280
_B8_H = 0.707106781186550
_BIOR15_8 = (
    (_B8_A,) * 8,
    (-_B8_B, -_B8_C, -_B8_C, -_B8_B, _B8_B, _B8_C, _B8_C, _B8_B),
    (_B8_D, _B8_E, -_B8_E, -_B8_D, -_B8_F, _B8_F, -_B8_F, _B8_F),
    (-_B8_F, _B8_F, -_B8_F, _B8_F, _B8_D, _B8_E, -_B8_E, -_B8_D),
    (_B8_H, -_B8_H, 0, 0, 0, 0, 0, 0),
    (0, 0, _B8_H, -_B8_H, 0, 0, 0, 0),
    (0, 0, 0, 0, _B8_H, -_B8_H, 0, 0),
    (0, 0, 0, 0, 0, 0, _B8_H, -_B8_H),
)


def dct_matrix(n: int) -> np.ndarray:
    """Orthonormal DCT-II, row = frequency (float64 formula, float32 storage)."""
    out = np.zeros((n, n), dtype=np.float32)
    for f in range(n):
        norm = np.sqrt(1.0 / n) if f == 0 else np.sqrt(2.0 / n)
        for s in range(n):
            out[f, s] = norm * np.cos(np.pi * (s + 0.5) * f / n)
    return out


def dst_matrix(n: int) -> np.ndarray:
    """DST-I with the reference's float32 index grids."""
    idx = np.arange(n, dtype=np.float32)
    col = idx.reshape((n, 1))
    return np.asarray(
        np.sqrt(2 / (n + 1)) * np.sin(np.pi * (col + 1) * (idx + 1) / (n + 1)),
        dtype=np.float32,
    )


def hadamard_matrix(n: int) -> np.ndarray:
    """Sylvester Hadamard matrix scaled by 1/sqrt(n) (n a power of two)."""
    if not (n and (n & (n - 1)) == 0):
        raise ValueError(f"Hadamard matrix size {n} must be a power of two.")
    h = np.ones((1, 1), dtype=np.float32)
    while h.shape[0] < n:
        h = np.block([[h, h], [h, -h]]).astype(np.float32)
    return h / np.float32(np.sqrt(n))


def haar_group_matrix(n: int) -> np.ndarray:
    """Hierarchical Haar matrix of a power-of-two group size, built in float32."""
    if not (n > 0 and (n & (n - 1)) == 0):
        raise ValueError(f"Haar group size must be a power of two, got {n}.")
    s = np.float32(1.0 / np.sqrt(2.0))
    m = np.ones((1, 1), dtype=np.float32)
    size = 1
    while size < n:
        coarse = np.kron(m, np.array([s, s], dtype=np.float32))
        detail = np.kron(np.eye(size, dtype=np.float32), np.array([s, -s], dtype=np.float32))
        m = np.vstack((coarse, detail)).astype(np.float32)
        size *= 2
    return m


def bior15_matrices(n: int) -> tuple[np.ndarray, np.ndarray]:
    """Tabulated bior1.5 analysis matrix and its inverse for n in {4, 8}."""
    if n == 4:
        fwd = np.array(_BIOR15_4, dtype=np.float32)
    elif n == 8:
        fwd = np.array(_BIOR15_8, dtype=np.float32)
    else:
        raise NotImplementedError(
            f"bior1.5 of length {n} needs PyWavelets filter banks; only lengths 4 and 8 "
            "are available on the GPU path."
        )
    inv = np.linalg.inv(fwd.astype(np.float64)).astype(np.float32)
    return fwd, inv


def axis_matrices(kind: TransformType, n: int) -> tuple[np.ndarray, np.ndarray]:
    """Forward and inverse matrices of one axis of length ``n``."""
    if kind is TransformType.DCT:
        f = dct_matrix(n)
        return f, np.ascontiguousarray(f.T)
    if kind is TransformType.DST:
        f = dst_matrix(n)
        # transforms.py builds the inverse from the transposed index grids
        idx = np.arange(n, dtype=np.float32)
        col = idx.reshape((n, 1))
        inv = np.asarray(
            np.sqrt(2 / (n + 1)) * np.sin(np.pi * (idx + 1) * (col + 1) / (n + 1)),
            dtype=np.float32,
        )
        return f, inv
    if kind is TransformType.HADAMARD:
        f = hadamard_matrix(n)
        return f, f
    if kind is TransformType.BIOR15:
        return bior15_matrices(n)
    raise NotImplementedError(f"transform {kind.name} is not available on the GPU path")


def resolve_axes(
    transform: Transform | list[Transform], ndim_patch: int
) -> tuple[str, list[TransformType | None]]:
    """Split a transform list into the group-axis kind and per-spatial-axis types.

    Mirrors get_transform_matrix (transforms.py:118-201): later entries override
    earlier ones on the axes they touch; ND covers every axis, GROUP axis 0,
    SPATIAL the patch axes.  Returns ``(group_kind, spatial_types)`` where
    ``group_kind`` is "haar", "dct" or "none".
    """
    items = [transform] if type(transform) is Transform else list(transform)
    group_kind = "none"
    spatial: list[TransformType | None] = [None] * ndim_patch
    for t in items:
        if t.type in (
            TransformType.STARLET,
            TransformType.ATROUS,
            TransformType.B3SPLINE,
            TransformType.CURVELET,
        ):
            raise NotImplementedError("operator transforms are not available on the GPU path")
        touches_group = t.mode in (TransformMode.ND, TransformMode.GROUP)
        touches_space = t.mode in (TransformMode.ND, TransformMode.SPATIAL)
        if touches_group:
            if t.type is TransformType.HAAR and t.mode is TransformMode.GROUP:
                group_kind = "haar"
            elif t.type is TransformType.DCT:
                group_kind = "dct"
            else:
                raise NotImplementedError(
                    f"group-axis transform {t.type.name}/{t.mode.name} is not available on the GPU path"
                )
        if touches_space:
            for a in range(ndim_patch):
                spatial[a] = t.type
    return group_kind, spatial
