"""Non-default Poisson options on the GPU vs the reference's own outputs.

Cases (``tests/golden/opt_*.npz``, made by ``make_golden.py option``): group-mass
conservation in both stages (2-D and 3-D) and in the hard-thresholding stage
only (ragged 2-D); the classic and noise-floor Wiener gains; the observation
as the Wiener variance source and as the Wiener matching source; soft
thresholding; the reference-finite-count and candidate-standardised HT match
policies; SSD matching with the Poisson noise-bias correction (gamma 3 and
2.5), whose distances the GPU evaluates in the reference's float32 operation
order, so its HT match sets must equal the reference's exactly.

Stated tolerance (as for the default Poisson pipeline): stage-1 match sets
equal the reference's except where the selection boundary is tied within the
reference's key rounding; both estimates within 1e-3 counts on at least 99.9%
of the voxels outside the footprint of groups whose match sets differ, and
PSNR within 0.01 dB of the reference's.
"""

import glob
import json
import os

import numpy as np
import pytest

from parity import compare_match_sets, output_parity, tie_footprint

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "opt_*.npz")))


def _profile(g):
    import bmnd_gb300 as bg

    cls = bg.BM3DProfile if str(g["kind"]) == "bm3d" else bg.BM4DProfile
    return cls(noise_model=bg.NoiseModel.POISSON, **json.loads(str(g["extra_json"])))


@pytest.mark.parametrize("case", CASES)
def test_option_pipeline_matches_reference(cuda, native, oracle_lib, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"opt_{case}.npz"))
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

    out = bg.bmnd(g["noisy"], profile, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    np.testing.assert_array_equal(out, stages["wiener"])
    shape = g["noisy"].shape
    blocks = {st: tuple(getattr(profile, f"{st}_block_size")) for st in ("ht", "wiener")}
    thr = float(np.float32(profile.ht_match_threshold))

    sel, cnt = matches["ht"]
    if profile.blockmatch_distance.value == "ssd":
        np.testing.assert_array_equal(cnt, g["ht_count"])
        np.testing.assert_array_equal(sel, g["ht_sel"])
    elif profile.poisson_ht_match_policy.value == "fixed":
        _, _, bad = compare_match_sets(oracle_lib, g["noisy"], blocks["ht"], g["ht_refs"], sel, cnt,
                                       g["ht_sel"], g["ht_count"], 1, thr)
        assert not bad, f"{case}/ht: unexplained match-set differences in groups {bad[:8]}"
    else:
        # per-reference thresholds or standardised distances: the oracle's tie
        # explanation does not apply; the match sets must still agree almost everywhere
        same = np.all(sel == g["ht_sel"], axis=1) & (cnt == g["ht_count"])
        assert same.mean() >= 0.97, (case, "ht match sets", same.mean())
    foot = tie_footprint(shape, blocks["ht"], sel, cnt, g["ht_sel"], g["ht_count"])
    par = output_parity(stages["ht"], g["ht"], g["clean"], exclude=foot)
    assert par["frac_within"] >= 0.999, (case, "ht", par)
    assert par["psnr_delta"] < 0.01, (case, "ht", par)

    sel, cnt = matches["wiener"]
    foot |= tie_footprint(shape, blocks["wiener"], sel, cnt, g["wiener_sel"], g["wiener_count"])
    par = output_parity(stages["wiener"], g["wiener"], g["clean"], exclude=foot)
    assert par["frac_within"] >= 0.999, (case, "wiener", par)
    assert par["psnr_delta"] < 0.01, (case, "wiener", par)


def test_mass_conservation_preserves_group_mass(cuda, native):
    """With conservation on, the estimate's normalised-occurrence-weighted mass
    over the stage equals the noisy mass it aggregates; without it, it does not
    in general.  Checked globally: sum(estimate) against the same functional of
    the input within 1e-3 relative."""
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, "opt_mass_bm3d_32.npz"))
    x = g["noisy"]
    with_mass = bg.bmnd(x, _profile(g))
    plain = bg.bmnd(x, bg.BM3DProfile(noise_model=bg.NoiseModel.POISSON))
    assert abs(float(with_mass.sum()) - float(x.sum())) <= 1e-3 * float(x.sum())
    assert not np.array_equal(with_mass, plain)
