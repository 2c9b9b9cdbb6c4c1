"""End-to-end GPU parity: bmnd() on the GPU vs the reference's own outputs and the oracle.

Stated tolerance:
* stage 1 (hard thresholding) match sets equal the reference's wherever the
  selection boundary is not tied within the reference's key rounding
  (parity.explain_mismatch);
* stage 2 (Wiener) matches on the pilot.  The GPU pilot accumulates in float64
  and differs from the reference's float32-accumulated pilot by ~1e-6
  relative, which moves real-valued distances across key quanta; the stage-2
  match sets are therefore checked against the oracle run on the GPU's own
  pilot (same rule), isolating the stage;
* estimates within 1e-3 counts on at least 99.9% of the voxels outside the
  footprint of tie-differing groups, and PSNR against the clean phantom
  within 0.01 dB of the reference's.
"""

import glob
import os

import numpy as np
import pytest

from parity import compare_match_sets, output_parity, tie_footprint

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "pipe_*.npz")))


def _profile(kind):
    import bmnd_gb300 as bg

    cls = bg.BM3DProfile if kind == "bm3d" else bg.BM4DProfile
    return cls(noise_model=bg.NoiseModel.POISSON)


@pytest.mark.parametrize("case", CASES)
def test_pipeline_matches_reference(cuda, native, oracle_lib, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"pipe_{case}.npz"))
    kind = str(g["kind"])
    profile = _profile(kind)
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

    out = bg.bmnd(g["noisy"], profile, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    assert out.dtype == np.float32 and out.shape == g["noisy"].shape
    np.testing.assert_array_equal(out, stages["wiener"])

    from bmnd_gb300 import plan
    from bmnd_gb300.validation import resolve_profile

    shape = g["noisy"].shape
    resolved = resolve_profile(_profile(kind), shape)
    thr = {st: float(np.float32(getattr(profile, f"{st}_match_threshold"))) for st in ("ht", "wiener")}
    blocks = {st: tuple(getattr(profile, f"{st}_block_size")) for st in ("ht", "wiener")}

    # stage 1 vs the reference itself
    sel, cnt = matches["ht"]
    eq, tied, bad = compare_match_sets(oracle_lib, g["noisy"], blocks["ht"], g["ht_refs"], sel, cnt,
                                       g["ht_sel"], g["ht_count"], 1, thr["ht"])
    assert not bad, f"{case}/ht: unexplained match-set differences in groups {bad[:8]}"
    ht_foot = tie_footprint(shape, blocks["ht"], sel, cnt, g["ht_sel"], g["ht_count"])

    # stage 2 vs the oracle on the GPU's own pilot
    pw = plan.stage_params(_profile(kind), shape, "wiener", resolved.blockmatch_distance, resolved.variance_k)
    o_est, o_sel, o_cnt, _ = oracle_lib.stage(pw, g["noisy"], stages["ht"], g["wiener_refs"])
    sel, cnt = matches["wiener"]
    eq, tied, bad = compare_match_sets(oracle_lib, stages["ht"], blocks["wiener"], g["wiener_refs"], sel, cnt,
                                       o_sel, o_cnt, 1, thr["wiener"])
    assert not bad, f"{case}/wiener: unexplained match-set differences in groups {bad[:8]}"
    w_foot = tie_footprint(shape, blocks["wiener"], sel, cnt, o_sel, o_cnt)
    par = output_parity(stages["wiener"], o_est, exclude=w_foot)
    assert par["frac_within"] >= 0.999, (case, "wiener-vs-oracle", par)

    # end to end vs the reference's estimates
    par = output_parity(stages["ht"], g["ht"], g["clean"], exclude=ht_foot)
    assert par["frac_within"] >= 0.999, (case, "ht", par)
    assert par["psnr_delta"] < 0.01, (case, "ht", par)
    sel, cnt = matches["wiener"]
    ref_foot = ht_foot | tie_footprint(shape, blocks["wiener"], sel, cnt, g["wiener_sel"], g["wiener_count"])
    par = output_parity(stages["wiener"], g["wiener"], g["clean"], exclude=ref_foot)
    assert par["frac_within"] >= 0.999, (case, "wiener", par)
    assert par["psnr_delta"] < 0.01, (case, "wiener", par)


@pytest.mark.parametrize("case", ["bm3d_64", "bm4d_16"])
def test_gpu_vs_oracle_stage_estimates(cuda, native, oracle_lib, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"pipe_{case}.npz"))
    profile = _profile(str(g["kind"]))
    stages = {}
    bg.bmnd(g["noisy"], profile, stage_callback=lambda s, e: stages.__setitem__(s, e))
    ref = oracle_lib.bmnd(g["noisy"], _profile(str(g["kind"])), return_details=True)[1]
    block = tuple(profile.ht_block_size)
    foot = tie_footprint(g["noisy"].shape, block, *_gpu_matches(bg, g["noisy"], profile)["ht"],
                         ref["ht"]["sel"], ref["ht"]["count"])
    par = output_parity(stages["ht"], ref["ht"]["estimate"], exclude=foot)
    assert par["frac_within"] >= 0.999, ("ht", par)
    # the oracle's Wiener stage runs on its own pilot; compare PSNR-level agreement
    par = output_parity(stages["wiener"], ref["wiener"]["estimate"], g["clean"])
    assert par["psnr_delta"] < 0.01, ("wiener", par)


def _gpu_matches(bg, noisy, profile):
    res = {}

    def cb(stage, result):
        k = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        sel = np.full((len(result.groups), k), -1, dtype=np.int32)
        cnt = np.zeros(len(result.groups), dtype=np.int32)
        for i, grp in enumerate(result.groups):
            sel[i, : grp.final_count] = grp.selected_lin_indices
            cnt[i] = grp.final_count
        res[stage] = (sel, cnt)

    bg.bmnd(noisy, profile, blockmatch_callback=cb)
    return res


def test_deterministic_and_input_forms(cuda, native):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, "pipe_bm3d_40x24.npz"))
    profile = _profile("bm3d")
    a = bg.bmnd(g["noisy"], profile)
    b = bg.bmnd(g["noisy"], profile)
    np.testing.assert_array_equal(a, b)
    # float64 input gives float32 output; non-contiguous input is accepted
    c = bg.bmnd(g["noisy"].astype(np.float64), profile)
    assert c.dtype == np.float32
    np.testing.assert_array_equal(a, c)
    big = np.zeros((80, 24), dtype=np.float32)
    big[::2] = g["noisy"]
    d = bg.bmnd(big[::2], profile)
    np.testing.assert_array_equal(a, d)
    # CUDA tensors in, CUDA tensor out
    t = bg.bmnd(cuda.from_numpy(g["noisy"]).cuda(), profile)
    assert t.is_cuda
    np.testing.assert_array_equal(a, t.cpu().numpy())


def test_zero_and_extreme_rates(cuda, native):
    import bmnd_gb300 as bg

    profile = _profile("bm3d")
    zero = np.zeros((24, 24), dtype=np.float32)
    out = bg.bmnd(zero, profile)
    assert np.array_equal(out, zero)
    rng = np.random.default_rng(0)
    for rate in (0.05, 5.0, 1e6):
        vol = rng.poisson(rate, size=(24, 24)).astype(np.float32)
        if not vol.any():
            vol[3, 3] = 1.0
        res = bg.bmnd(vol, _profile("bm3d"))
        assert np.all(np.isfinite(res))


@pytest.mark.parametrize("case", ["bm3d_32", "bm4d_12x16x20"])
def test_fast_haar_group_axis_matches_matrix_product(cuda, native, case):
    """The fast path's Haar group axis (sum pyramid) computes the same
    transform as the matrix product: both stages agree to float32 rounding."""
    import bmnd_gb300 as bg
    from bmnd_gb300.api import stage_device

    g = np.load(os.path.join(GOLDEN, f"pipe_{case}.npz"))
    profile = _profile(str(g["kind"]))
    x = cuda.from_numpy(g["noisy"]).cuda()
    for stage in ("ht", "wiener"):
        pilot = None if stage == "ht" else cuda.from_numpy(g["ht"]).cuda()
        a = stage_device(x, profile, stage, pilot).cpu().numpy()
        b = stage_device(x, profile, stage, pilot, fast_transforms=True).cpu().numpy()
        par = output_parity(b, a)
        assert par["frac_within"] >= 0.999, (case, stage, par)
    assert bg is not None
