"""return_sigma_map on the GPU against the reference's own sigma maps
(tests/golden/sigma_*.npz, generated by make_golden.py sigma)."""

import glob
import os

import numpy as np
import pytest

from parity import tie_footprint

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "sigma_*.npz")))


@pytest.mark.parametrize("case", CASES)
def test_sigma_maps_match_reference(cuda, native, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"sigma_{case}.npz"))
    kind = str(g["kind"])
    cls = bg.BM3DProfile if kind == "bm3d" else bg.BM4DProfile
    profile = cls(noise_model=bg.NoiseModel.POISSON)
    matches = {}

    def bm_cb(stage, result):
        k = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        sel = np.full((len(result.groups), k), -1, dtype=np.int32)
        cnt = np.zeros(len(result.groups), dtype=np.int32)
        for i, grp in enumerate(result.groups):
            sel[i, : grp.final_count] = grp.selected_lin_indices
            cnt[i] = grp.final_count
        matches[stage] = (sel, cnt)

    out, maps = bg.bmnd(g["noisy"], profile, return_sigma_map=True, blockmatch_callback=bm_cb)
    assert set(maps) == {"global", "ht", "wiener"}
    assert abs(maps["global"] - float(g["global_sigma"])) <= 1e-6 * float(g["global_sigma"])
    shape = g["noisy"].shape
    foot = np.zeros(shape, dtype=bool)
    for stage in ("ht", "wiener"):
        block = tuple(getattr(profile, f"{stage}_block_size"))
        foot |= tie_footprint(shape, block, *matches[stage], g[f"{stage}_sel"], g[f"{stage}_count"])
    for stage in ("ht", "wiener"):
        got, want = maps[stage], g[f"sigma_{stage}"]
        assert got.shape == want.shape and got.dtype == np.float32
        rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-6)
        keep = ~foot
        assert np.mean(rel[keep] <= 1e-3) >= 0.995, (stage, float(np.mean(rel[keep] <= 1e-3)))
        assert np.max(rel[keep]) < 5e-2, (stage, float(np.max(rel[keep])))


def test_sigma_map_zero_volume(cuda, native):
    import bmnd_gb300 as bg

    out, maps = bg.bmnd(np.zeros((24, 24), dtype=np.float32), bg.BM3DProfile(noise_model="poisson"),
                        return_sigma_map=True)
    assert set(maps) == {"ht", "wiener"} and not np.any(maps["ht"])
