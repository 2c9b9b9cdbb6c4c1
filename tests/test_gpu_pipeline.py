"""End-to-end GPU parity: bmnd() on the GPU vs the reference's own outputs and the oracle.

Stated tolerance (max abs error 1e-3 counts, PSNR within 0.01 dB):

* match sets: stage-1 sets equal the reference's, and stage-2 sets equal the
  oracle's on the GPU's own pilot, wherever the selection boundary is not
  tied within the reference's key rounding (``parity.explain_mismatch``);
* filtering, isolated: each stage of the oracle run on the GPU's own match
  sets (and, for Wiener, its pilot) gives the GPU stage estimate to within
  1e-3 counts at every voxel.  The float64 build of the oracle gives the
  per-stage error: the GPU (float64 aggregation) is no further from it than
  the reference's own float32 arithmetic (printed per stage);
* each stage against the oracle's own matching: within 1e-3 counts outside the
  footprint of groups whose match sets differ at ties;
* end to end against the reference's estimates: within 1e-3 counts outside the
  footprint of tie-differing groups (stage 2: and of the groups whose patches
  touch a voxel where the two pilots differ by more than 1e-3), PSNR against
  the clean phantom within 0.01 dB.

The same checks run on crops of the benchmark workloads: 96^3 of the 256^3
ellipsoid volume and 512^2 of the 2048^2 blob image (match sets on every
fourth reference, to bound the oracle's time).
"""

import glob
import os

import numpy as np
import pytest

from parity import (
    compare_match_sets,
    group_footprint,
    groups_touching,
    max_abs_outside,
    output_parity,
    tie_footprint,
)

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "pipe_*.npz")))
TOL = 1e-3


def _profile(kind):
    import bmnd_gb300 as bg

    cls = bg.BM3DProfile if kind == "bm3d" else bg.BM4DProfile
    return cls(noise_model=bg.NoiseModel.POISSON)


def _run_gpu(bg, noisy, profile):
    """bmnd() with both callbacks: stage estimates and match sets."""
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

    out = bg.bmnd(noisy, profile, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    return out, stages, matches


def _stage_setup(kind, shape, stage):
    from bmnd_gb300 import plan
    from bmnd_gb300.validation import resolve_profile

    prof = _profile(kind)
    resolved = resolve_profile(prof, shape)
    p = plan.stage_params(prof, shape, stage, resolved.blockmatch_distance, resolved.variance_k)
    block = tuple(getattr(prof, f"{stage}_block_size"))
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.ascontiguousarray(plan.reference_schedule(prof, counts, stage).reference_abs)
    thr = float(np.float32(getattr(prof, f"{stage}_match_threshold")))
    radius = tuple(getattr(prof, f"{stage}_search_window"))
    return p, block, refs, thr, radius


def _isolated_filtering(oracle_lib, tag, p, noisy, pilot, refs, sel, cnt, gpu_est):
    """The oracle's filtering on the GPU's match sets: max abs error against the
    float32 restatement, and the float64 per-stage error."""
    o32, _, _, _, marg = oracle_lib.stage(p, noisy, pilot, refs, sel=sel, count=cnt, margins=True)
    o64 = oracle_lib.stage(p, noisy, pilot, refs, sel=sel, count=cnt, f64=True)[0]
    err32 = max_abs_outside(gpu_est, o32)
    err_gpu64 = max_abs_outside(gpu_est, o64)
    err_ref64 = max_abs_outside(o32, o64)
    print(f"{tag}: max|gpu-oracle32|={err32:.3e} max|gpu-oracle64|={err_gpu64:.3e} "
          f"max|oracle32-oracle64|={err_ref64:.3e}")
    if err32 > TOL:
        # a hard-threshold decision within float32 rounding of its boundary
        # (relative margin <= 1e-5) may go either way in two float32
        # evaluations: outside those groups' footprint the bar holds, and
        # everywhere the GPU must stay within it of the float64 oracle
        block = tuple(int(p.block[a]) for a in range(p.ndim))
        near = np.flatnonzero(marg <= 1e-5)
        foot = group_footprint(noisy.shape, block, sel, cnt, near)
        err32_out = max_abs_outside(gpu_est, o32, foot)
        print(f"{tag}: {near.size} groups with a decision at its threshold; outside them "
              f"max|gpu-oracle32|={err32_out:.3e}")
        assert err32_out <= TOL, (tag, err32_out)
        assert err_gpu64 <= TOL, (tag, err_gpu64)
    assert err_gpu64 <= max(2.0 * err_ref64, 1e-5), (tag, err_gpu64, err_ref64)
    return o32


def _check_stages(oracle_lib, name, kind, noisy, stages, matches, ref_stride=1):
    """Match sets, isolated filtering and stage-vs-oracle checks of both stages."""
    shape = noisy.shape
    pilot = None
    for stage in ("ht", "wiener"):
        p, block, refs, thr, radius = _stage_setup(kind, shape, stage)
        sel, cnt = matches[stage]
        src = noisy if stage == "ht" else pilot
        # match sets against the oracle's (on the GPU's pilot for stage 2)
        idx = np.arange(0, len(refs), ref_stride)
        o_sel, o_cnt, _ = oracle_lib.blockmatch_volume(src, block, refs[idx], radius, p.max_stack, p.min_stack,
                                                       thr, 1)
        eq, tied, bad = compare_match_sets(oracle_lib, src, block, refs[idx], sel[idx], cnt[idx], o_sel, o_cnt,
                                           1, thr)
        assert not bad, f"{name}/{stage}: unexplained match-set differences in groups {idx[bad[:8]]}"
        # filtering on identical groups
        _isolated_filtering(oracle_lib, f"{name}/{stage}", p, noisy, pilot, refs, sel, cnt, stages[stage])
        pilot = stages[stage]


@pytest.mark.parametrize("case", CASES)
def test_pipeline_matches_reference(cuda, native, oracle_lib, case):
    import bmnd_gb300 as bg

    g = np.load(os.path.join(GOLDEN, f"pipe_{case}.npz"))
    kind = str(g["kind"])
    noisy = g["noisy"]
    shape = noisy.shape
    out, stages, matches = _run_gpu(bg, noisy, _profile(kind))
    assert out.dtype == np.float32 and out.shape == shape
    np.testing.assert_array_equal(out, stages["wiener"])

    _check_stages(oracle_lib, case, kind, noisy, stages, matches)

    # stage 1 end to end: match sets and estimate against the reference itself
    p, bh, refs, thr, _ = _stage_setup(kind, shape, "ht")
    sel, cnt = matches["ht"]
    eq, tied, bad = compare_match_sets(oracle_lib, noisy, bh, g["ht_refs"], sel, cnt, g["ht_sel"], g["ht_count"],
                                       1, thr)
    assert not bad, f"{case}/ht: unexplained match-set differences in groups {bad[:8]}"
    ht_foot = tie_footprint(shape, bh, sel, cnt, g["ht_sel"], g["ht_count"])
    err = max_abs_outside(stages["ht"], g["ht"], ht_foot)
    assert err <= TOL, (case, "ht", err)
    par = output_parity(stages["ht"], g["ht"], g["clean"])
    assert par["psnr_delta"] < 0.01, (case, "ht", par)

    # stage 2 against the oracle's own matching on the GPU pilot
    pw, bw, wrefs, wthr, _ = _stage_setup(kind, shape, "wiener")
    o_est, o_sel, o_cnt, _ = oracle_lib.stage(pw, noisy, stages["ht"], wrefs)
    wsel, wcnt = matches["wiener"]
    w_foot = tie_footprint(shape, bw, wsel, wcnt, o_sel, o_cnt)
    err = max_abs_outside(stages["wiener"], o_est, w_foot)
    assert err <= TOL, (case, "wiener-vs-oracle", err)

    # stage 2 end to end against the reference: outside the groups whose match
    # sets differ, and the groups that read a voxel where the pilots differ
    pilot_diff = np.abs(stages["ht"].astype(np.float64) - g["ht"]) > TOL
    rows = set(np.nonzero(~(np.all(wsel == g["wiener_sel"], axis=1) & (wcnt == g["wiener_count"])))[0])
    rows |= set(groups_touching(shape, bw, wsel, wcnt, pilot_diff))
    rows |= set(groups_touching(shape, bw, g["wiener_sel"], g["wiener_count"], pilot_diff))
    foot = group_footprint(shape, bw, wsel, wcnt, sorted(rows)) | group_footprint(
        shape, bw, g["wiener_sel"], g["wiener_count"], sorted(rows))
    err = max_abs_outside(stages["wiener"], g["wiener"], foot)
    assert err <= TOL, (case, "wiener", err)
    par = output_parity(stages["wiener"], g["wiener"], g["clean"])
    assert par["psnr_delta"] < 0.01, (case, "wiener", par)


@pytest.mark.parametrize("seed", range(1, 10))
def test_config1_seeds_against_oracle(cuda, native, oracle_lib, seed):
    """The 256^2 BM3D-Poisson configuration (12 rectangles and discs) on seeds
    1-9: the reference itself ran seed 0 (pipe_bm3d_256_cfg); the other seeds
    are checked against the oracle, which is pinned to that run (match sets on
    every fourth reference)."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms

    clean, noisy = phantoms.shapes_2d(256, seed=seed)
    out, stages, matches = _run_gpu(bg, noisy, _profile("bm3d"))
    _check_stages(oracle_lib, f"config1_seed{seed}", "bm3d", noisy, stages, matches, ref_stride=4)


@pytest.mark.parametrize("workload", ["bm4d256_crop96", "bm3d2048_crop512"])
def test_benchmark_workload_crop_parity(cuda, native, oracle_lib, workload):
    """The stage checks on crops of the benchmark volumes (256^3 ellipsoids,
    2048^2 blobs), at sizes the oracle finishes in seconds."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms

    if workload == "bm4d256_crop96":
        clean, noisy = phantoms.ellipsoids_3d(256, seed=0)
        sl = (slice(80, 176),) * 3
        kind = "bm4d"
    else:
        clean, noisy = phantoms.blobs_2d(2048, seed=0)
        sl = (slice(768, 1280),) * 2
        kind = "bm3d"
    noisy = np.ascontiguousarray(noisy[sl])
    clean = np.ascontiguousarray(clean[sl])
    out, stages, matches = _run_gpu(bg, noisy, _profile(kind))
    _check_stages(oracle_lib, workload, kind, noisy, stages, matches, ref_stride=4)
    # the oracle's own pipeline on the same crop: same quality
    ref = oracle_lib.bmnd(noisy, _profile(kind))
    par = output_parity(out, ref, clean)
    print(f"{workload}: PSNR gpu={par['psnr_out']:.4f} oracle={par['psnr_ref']:.4f} dB")
    assert par["psnr_delta"] < 0.01, par


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


@pytest.mark.parametrize("workload", ["bm4d128", "bm3d512"])
def test_bitwise_deterministic_at_size(cuda, native, workload):
    """Two runs give the same bits (the reference's property pinned by
    tests/test_bmnd_smoke.py:71): every voxel's sums have a fixed order, with no
    floating-point atomics, for the plain path and the learned fast path."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.pilot import PilotNet, bmnd_fast, default_net_path

    if workload == "bm4d128":
        _, noisy = phantoms.ellipsoids_3d(128, seed=5)
        kind = "bm4d"
    else:
        _, noisy = phantoms.blobs_2d(2048, seed=5)
        noisy = np.ascontiguousarray(noisy[:512, :512])
        kind = "bm3d"
    x = cuda.from_numpy(noisy).cuda()
    a = bg.bmnd_device(x, _profile(kind))
    b = bg.bmnd_device(x, _profile(kind))
    assert cuda.equal(a, b)
    net = PilotNet.load(default_net_path(kind))
    fa = bmnd_fast(x, _profile(kind), net)
    fb = bmnd_fast(x, _profile(kind), net)
    assert cuda.equal(fa, fb)
