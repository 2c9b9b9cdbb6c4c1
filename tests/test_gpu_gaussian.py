"""Stationary Gaussian noise on the GPU vs the reference's own outputs.

Cases (``tests/golden/gauss_*.npz``, made by ``make_golden.py gauss``): BM3D
with a scalar sigma, a ragged 2-D volume, sigma estimated from the data, a
coloured ``sigma_psd``, conventional mode (``nf=0``: no gamma correction,
k = 0), soft thresholding, a ragged BM4D volume, and group-scope
windowed-synthesis weights: with white noise the covariance-aware exact group
weighting (risk weights in the Wiener stage), with a coloured PSD the
diagonal weighting the reference falls back to (variance.py:1459-1470).

Stated tolerance:
* stage-1 match sets (SSD with the gamma noise-bias correction) equal the
  reference's in at least 95% of the groups and group sizes in at least 98%;
  differences come from candidates whose float32 distances tie within
  rounding;
* both stage estimates within 1e-3 x (max - min of the clean volume) on at
  least 99.9% of the voxels outside the footprint of groups whose match sets
  differ, and PSNR within 0.01 dB of the reference's;
* sigma maps within 1e-3 relative on the same voxels, and the same global
  sigma.
"""

import glob
import os

import numpy as np
import pytest

from parity import output_parity, tie_footprint

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "gauss_*.npz")))


def _profile(g):
    import json

    import bmnd_gb300 as bg

    if "extra_json" in g.files:
        extra = json.loads(str(g["extra_json"]))
    else:
        nf = int(g["nf"])
        extra = {} if nf < 0 else dict(nf=nf)
        if "soft" in g.files and int(g["soft"]):
            extra["ht_use_soft_thresholding"] = True
    return (bg.BM3DProfile if str(g["kind"]) == "bm3d" else bg.BM4DProfile)(**extra)


def _call(g):
    if "sigma_psd" in g.files:
        return dict(sigma_psd=g["sigma_psd"])
    s = float(g["sigma"])
    return {} if s < 0 else dict(sigma=s)


@pytest.mark.parametrize("case", CASES)
def test_gaussian_pipeline_matches_reference(cuda, native, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"gauss_{case}.npz"))
    profile = _profile(g)
    stages, matches = {}, {}

    def stage_cb(stage, est):
        stages[stage] = est

    def bm_cb(stage, result):
        k = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        sel = np.full((len(result.groups), k), -1, dtype=np.int32)
        cnt = np.zeros(len(result.groups), dtype=np.int32)
        for i, grp in enumerate(result.groups):
            sel[i, : grp.final_count] = grp.selected_lin_indices
            cnt[i] = grp.final_count
        matches[stage] = (sel, cnt)

    out, smap = bg.bmnd(g["noisy"], profile, return_sigma_map=True, stage_callback=stage_cb,
                        blockmatch_callback=bm_cb, **_call(g))
    assert out.dtype == np.float32 and out.shape == g["noisy"].shape
    np.testing.assert_array_equal(out, stages["wiener"])
    assert smap["global"] == pytest.approx(float(g["global_sigma"]), rel=1e-6)

    shape = g["noisy"].shape
    clean = g["clean"]
    tol = 1e-3 * float(clean.max() - clean.min())
    blocks = {st: tuple(getattr(profile, f"{st}_block_size")) for st in ("ht", "wiener")}

    sel, cnt = matches["ht"]
    same = np.all(sel == g["ht_sel"], axis=1) & (cnt == g["ht_count"])
    assert same.mean() >= 0.95, (case, "ht match sets", same.mean())
    assert np.mean(cnt == g["ht_count"]) >= 0.98
    foot = tie_footprint(shape, blocks["ht"], sel, cnt, g["ht_sel"], g["ht_count"])
    par = output_parity(stages["ht"], g["ht"], clean, tol=tol, exclude=foot)
    assert par["frac_within"] >= 0.999, (case, "ht", par)
    assert par["psnr_delta"] < 0.01, (case, "ht", par)

    sel, cnt = matches["wiener"]
    foot |= tie_footprint(shape, blocks["wiener"], sel, cnt, g["wiener_sel"], g["wiener_count"])
    par = output_parity(stages["wiener"], g["wiener"], clean, tol=tol, exclude=foot)
    assert par["frac_within"] >= 0.999, (case, "wiener", par)
    assert par["psnr_delta"] < 0.01, (case, "wiener", par)

    for stage in ("ht", "wiener"):
        got, want = np.asarray(smap[stage], np.float64), g[f"sigma_{stage}"].astype(np.float64)
        keep = ~foot
        rel = np.abs(got - want)[keep] / np.maximum(np.abs(want[keep]), 1e-12)
        assert np.mean(rel <= 1e-3) >= 0.999, (case, stage, float(np.max(rel)))


def test_gaussian_device_input_and_negative_values(cuda, native):
    """CUDA-tensor input stays on the device; negative values are valid for Gaussian noise."""
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, "gauss_bm3d_32.npz"))
    x = g["noisy"] - np.float32(10.0)
    host = bg.bmnd(x, bg.BM3DProfile(), sigma=3.0)
    dev = bg.bmnd(cuda.from_numpy(x).cuda(), bg.BM3DProfile(), sigma=3.0)
    assert dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    # the matching and the noise model are offset-invariant; the Wiener gain of
    # the group DC is not, so only the denoising quality is compared
    base = bg.bmnd(g["noisy"], bg.BM3DProfile(), sigma=3.0)
    clean = g["clean"].astype(np.float64)
    err_base = np.sqrt(np.mean((base - clean) ** 2))
    err_shift = np.sqrt(np.mean((host + 10.0 - clean) ** 2))
    assert np.all(np.isfinite(host)) and abs(err_shift - err_base) < 0.05 * err_base
