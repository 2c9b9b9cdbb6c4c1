"""The C oracle against the reference's own outputs (golden fixtures), on CPU.

Pins the oracle before it is trusted as the GPU checker: same schedules, same
match sets (up to near-ties of the reference's key rounding), estimates
within 1e-3 counts of the reference everywhere outside tie footprints.
"""

import glob
import os

import numpy as np
import pytest

from parity import compare_match_sets, output_parity, tie_footprint

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "pipe_*.npz")))
UNIT = os.path.join(GOLDEN, "unit_reference.npz")


def _profile(kind):
    import bmnd_gb300 as bg

    cls = bg.BM3DProfile if kind == "bm3d" else bg.BM4DProfile
    return cls(noise_model=bg.NoiseModel.POISSON)


@pytest.mark.parametrize("case", CASES)
def test_oracle_pipeline_matches_reference(oracle_lib, case):
    """Stage 1 on the noisy input, stage 2 on the reference's own pilot (so a
    near-tie in stage 1 cannot move stage 2's match sets)."""
    from bmnd_gb300 import plan
    from bmnd_gb300.validation import resolve_profile

    g = np.load(os.path.join(GOLDEN, f"pipe_{case}.npz"))
    kind = str(g["kind"])
    profile = _profile(kind)
    shape = g["noisy"].shape
    resolved = resolve_profile(_profile(kind), shape)
    for stage in ("ht", "wiener"):
        params = plan.stage_params(profile, shape, stage, resolved.blockmatch_distance, resolved.variance_k)
        refs = g[f"{stage}_refs"].astype(np.int32)
        pilot = None if stage == "ht" else g["ht"]
        est, sel, cnt, _ = oracle_lib.stage(params, g["noisy"], pilot, refs)
        src = g["noisy"] if stage == "ht" else g["ht"]
        block = tuple(getattr(profile, f"{stage}_block_size"))
        thr = float(np.float32(getattr(profile, f"{stage}_match_threshold")))
        eq, tied, bad = compare_match_sets(oracle_lib, src, block, refs, sel, cnt,
                                           g[f"{stage}_sel"], g[f"{stage}_count"], 1, thr)
        assert not bad, (case, stage, bad[:8])
        assert eq >= 0.98 * len(cnt)
        foot = tie_footprint(shape, block, sel, cnt, g[f"{stage}_sel"], g[f"{stage}_count"])
        par = output_parity(est, g[stage], g["clean"], exclude=foot)
        assert par["frac_within"] >= 0.999 and par["psnr_delta"] < 0.01, (stage, par)


def test_oracle_schedule_and_full_pipeline(oracle_lib):
    """The oracle's own two-stage run reproduces the reference's schedules and
    its final PSNR on the 256 x 256 configuration."""
    g = np.load(os.path.join(GOLDEN, "pipe_bm3d_256_cfg.npz"))
    out, det = oracle_lib.bmnd(g["noisy"], _profile("bm3d"), return_details=True)
    for stage in ("ht", "wiener"):
        np.testing.assert_array_equal(det[stage]["refs"], g[f"{stage}_refs"])
    from bmnd_gb300.phantoms import psnr

    assert abs(psnr(out, g["clean"]) - psnr(g["wiener"], g["clean"])) < 0.01


def test_oracle_distances_match_reference(oracle_lib):
    u = np.load(UNIT)
    for pv in (64, 125):
        ref_p, cand = u[f"dist_p{pv}_ref"], u[f"dist_p{pv}_cand"]
        for code in range(4):
            want = u[f"dist_p{pv}_c{code}"]
            got = np.array([oracle_lib.patch_distance(ref_p[i], cand[i], code) for i in range(len(want))],
                           dtype=np.float32)
            rel = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-6)
            # float32 sums with different log implementations: a few ulp of the sum
            assert np.max(rel) < 2e-5, (pv, code, float(np.max(rel)))
            if code in (0, 2, 3):
                assert np.mean(got == want) > 0.95, (pv, code)


def test_canonical_keys_exact(oracle_lib):
    u = np.load(UNIT)
    got = oracle_lib.canonical(u["canon_in"])
    np.testing.assert_array_equal(got, u["canon_out"])


@pytest.mark.parametrize("idx", range(6))
def test_oracle_schedule_matches_reference(oracle_lib, idx):
    u = np.load(UNIT)
    a, sh, sf = oracle_lib.schedule(tuple(u[f"sched{idx}_counts"]), tuple(u[f"sched{idx}_block"]),
                                    tuple(u[f"sched{idx}_step"]))
    np.testing.assert_array_equal(a, u[f"sched{idx}_abs"])
    np.testing.assert_array_equal(sh, u[f"sched{idx}_shifted"])
    np.testing.assert_array_equal(sf, u[f"sched{idx}_shift"])


def test_oracle_poisson_ssd_bias_known_answer(oracle_lib):
    # tests/test_blockmatching_internal_unit.py:203-229: patches [0] and [2],
    # threshold 1; gamma 2 times the bias 1 * (0 + 2) brings the SSD 4 to 0
    vol = np.array([0.0, 2.0], dtype=np.float32)
    sel, cnt, _ = oracle_lib.blockmatch_volume_poisson_biased(vol, (1,), [[0]], (1,), 2, 1, 1.0, 0.0, pow2=False)
    assert sel[0, : cnt[0]].tolist() == [0]
    sel, cnt, acc = oracle_lib.blockmatch_volume_poisson_biased(vol, (1,), [[0]], (1,), 2, 1, 1.0, 2.0,
                                                                pow2=False)
    assert sel[0, : cnt[0]].tolist() == [0, 1] and acc[0] == 2


@pytest.mark.parametrize("case", ["ssd_gamma_bm3d_32", "ssd_gamma_bm4d_12x16x20"])
def test_oracle_poisson_ssd_bias_matches_reference(oracle_lib, case):
    """The oracle's SSD matching with the Poisson noise bias reproduces the
    reference's stage-1 match sets exactly (threshold float32(t (max - min)^2)
    over the noisy volume, blockmatching.py:168-184)."""
    import json

    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"opt_{case}.npz"))
    cls = bg.BM3DProfile if str(g["kind"]) == "bm3d" else bg.BM4DProfile
    profile = cls(noise_model=bg.NoiseModel.POISSON, **json.loads(str(g["extra_json"])))
    noisy = g["noisy"]
    d = np.float32(noisy.max()) - np.float32(noisy.min())
    thr = np.float32(float(profile.ht_match_threshold) * float(d) * float(d))
    sel, cnt, acc = oracle_lib.blockmatch_volume_poisson_biased(
        noisy, tuple(profile.ht_block_size), g["ht_refs"], tuple(profile.ht_search_window),
        int(profile.ht_max_stack_size), int(profile.ht_min_stack_size), thr, float(profile.gamma),
        count_scale=float(profile.poisson_count_scale))
    np.testing.assert_array_equal(cnt, g["ht_count"])
    np.testing.assert_array_equal(sel, g["ht_sel"])
    np.testing.assert_array_equal(acc, g["ht_accepted"])
