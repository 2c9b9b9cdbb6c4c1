"""Parity helpers shared by the tests.

Match sets: the reference orders candidates by canonical distance keys whose
quantum is 2^-18 * 2^floor(log2 max(d, 1)) (src/bmnd/blockmatching.py:957-964).
Two correct float32 evaluations of the same distance (different log
implementations, different accumulation) can land in adjacent quanta, so a
selected set may differ where two candidates are tied to within that
rounding.  ``explain_mismatch`` accepts a differing row only if every swapped
candidate pair is tied to within ``TIE_QUANTA`` quanta of their float64
distances, or the difference is a candidate within the same margin of the
threshold.
"""

from __future__ import annotations

import numpy as np

TIE_QUANTA = 4.0


def quantum(d: float) -> float:
    mag = max(abs(float(d)), 1.0)
    return 2.0 ** (np.floor(np.log2(mag)) - 18)


def unravel(lin: int, counts) -> tuple[int, ...]:
    out = []
    for c in reversed(counts):
        out.append(lin % c)
        lin //= c
    return tuple(reversed(out))


def patch_at(volume: np.ndarray, block, lin: int) -> np.ndarray:
    counts = tuple(s - b + 1 for s, b in zip(volume.shape, block))
    q = unravel(int(lin), counts)
    sl = tuple(slice(a, a + b) for a, b in zip(q, block))
    return np.ascontiguousarray(volume[sl], dtype=np.float32).reshape(-1)


def explain_mismatch(oracle, volume, block, ref_pos, row_a, row_b, code, threshold, count_scale=1.0):
    """True if rows a and b differ only by near-tied candidates."""
    counts = tuple(s - b + 1 for s, b in zip(volume.shape, block))
    ref_lin = int(np.ravel_multi_index(tuple(int(x) for x in ref_pos), counts))
    ref_patch = patch_at(volume, block, ref_lin)
    set_a = {int(x) for x in row_a if x >= 0}
    set_b = {int(x) for x in row_b if x >= 0}
    only_a, only_b = set_a - set_b, set_b - set_a
    if not only_a and not only_b:
        return True  # same members, order differs only among ties (checked by caller if needed)

    def d64(lin):
        return oracle.patch_distance(ref_patch, patch_at(volume, block, lin), code, count_scale, f64=True)

    da = [d64(x) for x in only_a]
    db = [d64(x) for x in only_b]
    # both sides non-empty: the boundary members must be tied
    if da and db:
        for x in da:
            for y in db:
                if abs(x - y) > TIE_QUANTA * quantum(max(x, y)):
                    return False
        return True
    # one side longer: the extra members sit at the threshold (accept/reject flip)
    extra = da or db
    return all(abs(x - threshold) <= TIE_QUANTA * quantum(max(x, threshold)) for x in extra)


def compare_match_sets(oracle, volume, block, refs, sel_a, cnt_a, sel_b, cnt_b, code, threshold,
                       count_scale=1.0):
    """Return (n_equal_rows, n_tied_rows, list of unexplained row indices)."""
    equal = np.all(sel_a == sel_b, axis=1) & (cnt_a == cnt_b)
    bad = []
    tied = 0
    for i in np.nonzero(~equal)[0]:
        if explain_mismatch(oracle, volume, block, refs[i], sel_a[i, : cnt_a[i]], sel_b[i, : cnt_b[i]],
                            code, threshold, count_scale):
            tied += 1
        else:
            bad.append(int(i))
    return int(equal.sum()), tied, bad


def psnr(x, ref, peak):
    mse = float(np.mean((np.asarray(x, np.float64) - np.asarray(ref, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(peak * peak / mse)


def tie_footprint(shape, block, sel_a, cnt_a, sel_b, cnt_b):
    """Voxels covered by any patch of a group whose two match sets differ."""
    mask = np.zeros(shape, dtype=bool)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    rows = np.nonzero(~(np.all(sel_a == sel_b, axis=1) & (cnt_a == cnt_b)))[0]
    for i in rows:
        for lin in list(sel_a[i, : cnt_a[i]]) + list(sel_b[i, : cnt_b[i]]):
            q = unravel(int(lin), counts)
            mask[tuple(slice(a, a + b) for a, b in zip(q, block))] = True
    return mask


def output_parity(out, ref, clean=None, tol=1e-3, exclude=None):
    """Dict of agreement figures between two denoised volumes.

    ``exclude`` masks voxels whose estimate legitimately differs (footprint of
    near-tied groups); ``frac_within`` is taken over the remaining voxels.
    """
    diff = np.abs(np.asarray(out, np.float64) - np.asarray(ref, np.float64))
    keep = np.ones(diff.shape, dtype=bool) if exclude is None else ~exclude
    res = {
        "max_abs": float(diff.max()),
        "frac_within": float(np.mean(diff[keep] <= tol)) if keep.any() else 1.0,
        "tie_voxels": int((~keep).sum()),
    }
    if clean is not None:
        peak = float(np.max(clean))
        res["psnr_out"] = psnr(out, clean, peak)
        res["psnr_ref"] = psnr(ref, clean, peak)
        res["psnr_delta"] = abs(res["psnr_out"] - res["psnr_ref"])
    return res


def group_footprint(shape, block, sel, cnt, rows):
    """Voxels covered by the patches of the given groups."""
    mask = np.zeros(shape, dtype=bool)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    for i in rows:
        for lin in sel[i, : cnt[i]]:
            q = unravel(int(lin), counts)
            mask[tuple(slice(a, a + b) for a, b in zip(q, block))] = True
    return mask


def groups_touching(shape, block, sel, cnt, mask):
    """Indices of the groups with a patch that overlaps ``mask``."""
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    rows = []
    for i in range(len(cnt)):
        for lin in sel[i, : cnt[i]]:
            q = unravel(int(lin), counts)
            if mask[tuple(slice(a, a + b) for a, b in zip(q, block))].any():
                rows.append(i)
                break
    return rows


def max_abs_outside(a, b, exclude=None) -> float:
    """Largest |a - b| over the voxels outside ``exclude`` (0 if none remain)."""
    diff = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    if exclude is not None:
        diff = diff[~exclude]
    return float(diff.max()) if diff.size else 0.0
