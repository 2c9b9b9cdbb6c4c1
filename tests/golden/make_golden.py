"""Generate the golden fixtures under ``tests/golden/`` from the reference itself.

The reference (cduhme/bmnd, pure Python + Numba) is imported from its source
tree with the import stand-ins in ``oracle/shim`` (``numba.njit`` = identity,
``pywt.Wavelet`` metadata only), so every loop runs with NumPy float32
semantics.  The fixtures are committed; this script is only needed to
regenerate them and needs the reference checkout, which the GPU machines do
not have.

Usage (``BMND_REFERENCE_SRC`` names the reference's ``src/`` directory)::

    BMND_REFERENCE_SRC=<reference>/src python tests/golden/make_golden.py unit
    python tests/golden/make_golden.py pipeline bm3d_32 [bm4d_16 ...]
    python tests/golden/make_golden.py sigma bm3d_32 [bm4d_12x16x20 ...]
    python tests/golden/make_golden.py gauss [bm3d_32 ...]
    python tests/golden/make_golden.py option [mass_bm3d_32 ...]
    python tests/golden/make_golden.py exact_risk
    python tests/golden/make_golden.py list

``unit`` writes ``unit_*.npz`` (distances, canonical keys, transforms, exact
and approximate Poisson sigma, weights, schedules); ``pipeline`` writes
``pipe_<case>.npz`` with the noisy input, both stage estimates (via
``stage_callback``) and both stages' match sets (via ``blockmatch_callback``).
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE_SRC = os.environ.get("BMND_REFERENCE_SRC")
if not REFERENCE_SRC or not os.path.isdir(REFERENCE_SRC):
    sys.exit("set BMND_REFERENCE_SRC to the reference package's src/ directory (the one holding bmnd/)")
sys.dont_write_bytecode = True
sys.path.insert(0, os.path.join(REPO, "oracle", "shim"))
sys.path.insert(1, REFERENCE_SRC)
sys.path.insert(2, REPO)

from bmnd_gb300 import phantoms  # noqa: E402

# name -> (profile kind, generator, kwargs, extra profile fields)
PIPELINE_CASES = {
    "bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=1), {}),
    "bm3d_48": ("bm3d", phantoms.shapes_2d, dict(size=48, seed=2), {}),
    "bm3d_64": ("bm3d", phantoms.shapes_2d, dict(size=64, seed=3), {}),
    "bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=6), {}),
    "bm3d_lowcount_32": ("bm3d", "lowcount2d", dict(size=32, seed=7), {}),
    "bm4d_16": ("bm4d", phantoms.ellipsoids_3d, dict(size=16, seed=4, count=6), {}),
    "bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=5), {}),
    "bm3d_256_cfg": ("bm3d", phantoms.shapes_2d, dict(size=256, seed=0), {}),
}


def _make_input(gen, kwargs):
    if gen == "ragged2d":
        shape = kwargs["shape"]
        clean, _ = phantoms.shapes_2d(size=max(shape), seed=kwargs["seed"])
        clean = np.ascontiguousarray(clean[: shape[0], : shape[1]])
        return clean, phantoms.poisson_noise(clean, kwargs["seed"])
    if gen == "lowcount2d":
        clean, _ = phantoms.shapes_2d(size=kwargs["size"], seed=kwargs["seed"])
        clean = clean * np.float32(2.0 / float(clean.max()))
        return clean, phantoms.poisson_noise(clean, kwargs["seed"])
    if gen == "ragged3d":
        shape = kwargs["shape"]
        clean, _ = phantoms.ellipsoids_3d(size=shape, seed=kwargs["seed"], count=6)
        return clean, phantoms.poisson_noise(clean, kwargs["seed"])
    return gen(**kwargs)


def _pack_matches(result, max_stack, ndim):
    groups = result.groups
    n = len(groups)
    sel = np.full((n, max_stack), -1, dtype=np.int32)
    counts = np.zeros(n, dtype=np.int32)
    accepted = np.zeros(n, dtype=np.int32)
    refs = np.zeros((n, ndim), dtype=np.int32)
    for i, group in enumerate(groups):
        k = int(group.final_count)
        sel[i, :k] = group.selected_lin_indices[:k]
        counts[i] = k
        accepted[i] = int(group.accepted_count)
        refs[i] = group.reference_abs
    return sel, counts, accepted, refs


def run_pipeline(name: str) -> None:
    import bmnd as ref

    kind, gen, kwargs, extra = PIPELINE_CASES[name]
    clean, noisy = _make_input(gen, kwargs)
    profile_cls = ref.BM3DProfile if kind == "bm3d" else ref.BM4DProfile
    profile = profile_cls(noise_model=ref.NoiseModel.POISSON, **extra)
    stages = {}
    matches = {}

    def stage_cb(stage, est):
        stages[stage] = np.asarray(est, dtype=np.float32)

    def bm_cb(stage, result):
        max_stack = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        matches[stage] = _pack_matches(result, max_stack, noisy.ndim)

    t0 = time.time()
    out = ref.bmnd(noisy, profile, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    elapsed = time.time() - t0
    payload = dict(
        kind=np.array(kind),
        clean=clean,
        noisy=noisy,
        ht=stages["ht"],
        wiener=stages["wiener"],
        out=np.asarray(out, dtype=np.float32),
        seconds=np.float64(elapsed),
    )
    for stage, (sel, counts, accepted, refs) in matches.items():
        payload[f"{stage}_sel"] = sel
        payload[f"{stage}_count"] = counts
        payload[f"{stage}_accepted"] = accepted
        payload[f"{stage}_refs"] = refs
    path = os.path.join(HERE, f"pipe_{name}.npz")
    np.savez_compressed(path, **payload)
    print(f"{name}: {noisy.shape} in {elapsed:.1f} s -> {path}")


def run_sigma(name: str) -> None:
    """sigma_<case>.npz: the reference's return_sigma_map output (global value and
    both stages' maps), with the stage estimates and match sets of the same run."""
    import bmnd as ref

    kind, gen, kwargs, extra = PIPELINE_CASES[name]
    clean, noisy = _make_input(gen, kwargs)
    profile_cls = ref.BM3DProfile if kind == "bm3d" else ref.BM4DProfile
    profile = profile_cls(noise_model=ref.NoiseModel.POISSON, **extra)
    stages, matches = {}, {}

    def stage_cb(stage, est):
        stages[stage] = np.asarray(est, dtype=np.float32)

    def bm_cb(stage, result):
        max_stack = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        matches[stage] = _pack_matches(result, max_stack, noisy.ndim)

    t0 = time.time()
    out, smap = ref.bmnd(noisy, profile, return_sigma_map=True, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    elapsed = time.time() - t0
    payload = dict(kind=np.array(kind), clean=clean, noisy=noisy, ht=stages["ht"], wiener=stages["wiener"],
                   out=np.asarray(out, dtype=np.float32), global_sigma=np.float64(smap["global"]),
                   sigma_ht=np.asarray(smap["ht"], dtype=np.float32),
                   sigma_wiener=np.asarray(smap["wiener"], dtype=np.float32), seconds=np.float64(elapsed))
    for stage, (sel, counts, accepted, refs) in matches.items():
        payload[f"{stage}_sel"] = sel
        payload[f"{stage}_count"] = counts
        payload[f"{stage}_refs"] = refs
    path = os.path.join(HERE, f"sigma_{name}.npz")
    np.savez_compressed(path, **payload)
    print(f"sigma {name}: {noisy.shape} in {elapsed:.1f} s -> {path}")


def run_unit() -> None:
    from bmnd import blockmatching as bm
    from bmnd import shifts, transforms, utils, variance, aggregationweights, wiener, poisson
    from bmnd.enums import AggregationWeightDomain, AggregationWeightModel, AggregationWeightScope
    from bmnd.profiles import BM3DProfile, BM4DProfile

    rng = np.random.default_rng(1234)
    out = {}

    # --- patch distances and canonical keys (all four distance codes) ---
    for patch_vol in (64, 125):
        n_pairs = 1000
        lam = rng.uniform(0.0, 60.0, size=(n_pairs, 1))
        ref_p = rng.poisson(lam, size=(n_pairs, patch_vol)).astype(np.float32)
        cand = rng.poisson(lam * rng.uniform(0.6, 1.4, size=(n_pairs, 1)), size=(n_pairs, patch_vol)).astype(np.float32)
        # a share of real-valued (pilot-like) patches
        ref_p[: n_pairs // 3] += rng.uniform(0.0, 1.0, size=(n_pairs // 3, patch_vol)).astype(np.float32)
        cand[: n_pairs // 3] += rng.uniform(0.0, 1.0, size=(n_pairs // 3, patch_vol)).astype(np.float32)
        # zero patches and identical pairs
        ref_p[-20:] = 0.0
        cand[-40:-20] = ref_p[-40:-20]
        for code in range(4):
            d = np.array(
                [bm._patch_distance_numba(ref_p[i], cand[i], code, 1.0) for i in range(n_pairs)],
                dtype=np.float32,
            )
            out[f"dist_p{patch_vol}_c{code}"] = d
        out[f"dist_p{patch_vol}_ref"] = ref_p
        out[f"dist_p{patch_vol}_cand"] = cand
    keys_in = np.concatenate(
        [
            rng.uniform(0.0, 1.0, 2000),
            rng.uniform(1.0, 8.0, 2000),
            rng.uniform(8.0, 1e4, 1000),
            np.array([0.0, 1.0, 2.0, 2.9527, 0.3937, 0.7689, 3.0, 4.0 - 1e-6]),
        ]
    ).astype(np.float32)
    out["canon_in"] = keys_in
    out["canon_out"] = np.array([bm._canonicalize_poisson_distance_numba(np.float32(v)) for v in keys_in], dtype=np.float32)

    # --- transforms ---
    for n in (4, 8):
        f, i = transforms.get_transform_matrix((1, n), [transforms.Transform(transforms.TransformType.BIOR15, transforms.TransformMode.SPATIAL)])
        out[f"bior15_fwd_{n}"] = np.asarray(f[1], dtype=np.float32)
        out[f"bior15_inv_{n}"] = np.asarray(i[1], dtype=np.float32)
    for n in (4, 5, 8):
        f, i = transforms.get_transform_matrix((1, n), [transforms.Transform(transforms.TransformType.DCT, transforms.TransformMode.SPATIAL)])
        out[f"dct_fwd_{n}"] = np.asarray(f[1], dtype=np.float32)
        out[f"dct_inv_{n}"] = np.asarray(i[1], dtype=np.float32)
    for n in (1, 2, 4, 8, 16, 32, 3, 6):
        f, i = transforms.get_transform_matrix((n, 4), [transforms.Transform(transforms.TransformType.HAAR, transforms.TransformMode.GROUP)])
        out[f"haar_fwd_{n}"] = np.asarray(f[0], dtype=np.float32)
        out[f"haar_inv_{n}"] = np.asarray(i[0], dtype=np.float32)
    for shape in ((8, 8), (4, 4, 4), (5, 5, 5)):
        out["kaiser_" + "x".join(map(str, shape))] = utils.kaiser_window_nd(shape, beta=2.0)

    # --- schedules (GENERATED, defaults) ---
    sched_cases = [
        ((25, 25), (8, 8), (3, 3)),
        ((17, 41), (8, 8), (3, 3)),
        ((249, 249), (8, 8), (3, 3)),
        ((13, 13, 13), (4, 4, 4), (3, 3, 3)),
        ((9, 13, 17), (5, 5, 5), (3, 3, 3)),
        ((1, 7), (8, 8), (3, 3)),
    ]
    for idx, (counts, block, step) in enumerate(sched_cases):
        items = shifts.get_reference_schedule(counts, block, step, mode="generated", shift_density=2.0, schedule_density=2)
        out[f"sched{idx}_counts"] = np.array(counts, dtype=np.int64)
        out[f"sched{idx}_block"] = np.array(block, dtype=np.int64)
        out[f"sched{idx}_step"] = np.array(step, dtype=np.int64)
        out[f"sched{idx}_abs"] = np.array([it.reference_abs for it in items], dtype=np.int64).reshape(-1, len(counts))
        out[f"sched{idx}_shifted"] = np.array([it.reference_shifted for it in items], dtype=np.int64).reshape(-1, len(counts))
        out[f"sched{idx}_shift"] = np.array([it.shift for it in items], dtype=np.int64).reshape(-1, len(counts))

    # --- group filtering pieces: approximate and exact Poisson sigma, weights, gains ---
    cases = [
        ("ht2d", BM3DProfile().ht_transform, (8, 8), 16, 19),
        ("wi2d", BM3DProfile().wiener_transform, (8, 8), 32, 19),
        ("ht3d", BM4DProfile().ht_transform, (4, 4, 4), 16, 7),
        ("wi3d", BM4DProfile().wiener_transform, (5, 5, 5), 32, 7),
    ]
    for tag, tlist, block, nmax, radius in cases:
        ndim = len(block)
        vol_shape = tuple(b + 2 * radius + 3 for b in block)
        vol = rng.poisson(20.0, size=vol_shape).astype(np.float32)
        vmodel = variance.build_poisson_variance_model(vol, variance_floor=1e-10, scale=1.0, source_name="observation")
        counts = tuple(s - b + 1 for s, b in zip(vol_shape, block))
        for n in sorted({1, 2, 4, 8, nmax}):
            if n > nmax:
                continue
            # random distinct positions in the counts grid, clustered to create overlap
            lin = rng.choice(int(np.prod(counts)), size=n, replace=False)
            abs_pos = np.array(np.unravel_index(lin, counts)).T.astype(np.int64)
            shifted = abs_pos - abs_pos.min(axis=0, keepdims=True)
            group_shape = (n,) + block
            fwd, inv = transforms.get_transform_matrix(group_shape, tlist)
            patches = np.stack([vol[tuple(slice(a, a + b) for a, b in zip(p, block))] for p in abs_pos])
            vpatches = np.stack([vmodel.variance_volume[tuple(slice(a, a + b) for a, b in zip(p, block))] for p in abs_pos])
            coef = transforms.apply_transform_nd(patches, fwd)
            sigma_approx = variance.get_direct_poisson_noise_std(vpatches, fwd, k=0)
            sigma = variance.get_direct_poisson_noise_std(
                vpatches, fwd, k=4, variance_model=vmodel,
                selected_abs_positions=abs_pos, selected_shifted_positions=shifted, group_shape=group_shape,
            )
            thr = np.float32(3.0) * sigma
            mask = poisson._poisson_hard_threshold_mask(np.abs(coef), thr, 1.0)
            w_patch = utils.kaiser_window_nd(block, beta=2.0)
            metric = aggregationweights.get_synthesis_risk_metric_factors(group_shape, inv, w_patch)
            att = np.asarray(mask, dtype=np.float32)
            weights_ht = aggregationweights.compute_aggregation_weights(
                att, model=AggregationWeightModel.VARIANCE, domain=AggregationWeightDomain.COEFFICIENT,
                scope=AggregationWeightScope.PATCH, noise_variance=np.asarray(sigma, dtype=np.float32) ** 2,
                signal_power=None, inverse_transform=inv, w_patch=w_patch, metric_factors=metric,
                mass_functional=None, eps=1e-10,
            )
            filt = transforms.apply_transform_nd(coef * mask, inv)
            gain = wiener.compute_poisson_wiener_gain(coef, sigma, 0.4, eps=1e-10)
            key = f"grp_{tag}_n{n}"
            out[key + "_vol"] = vol
            out[key + "_abs"] = abs_pos
            out[key + "_coef"] = np.asarray(coef, dtype=np.float32)
            out[key + "_sigma_approx"] = sigma_approx
            out[key + "_sigma"] = np.asarray(sigma, dtype=np.float32)
            out[key + "_mask"] = np.asarray(mask, dtype=np.uint8)
            out[key + "_weights_ht"] = np.asarray(weights_ht, dtype=np.float32)
            out[key + "_filt_ht"] = np.asarray(filt, dtype=np.float32)
            out[key + "_gain"] = np.asarray(gain, dtype=np.float32)

    path = os.path.join(HERE, "unit_reference.npz")
    np.savez_compressed(path, **out)
    print(f"unit fixtures -> {path} ({len(out)} arrays)")


def run_exact_risk() -> None:
    """exact_risk_groups.npz: the covariance-aware exact group weighting on
    single groups, made by the reference's own functions
    (build_exact_poisson_group_plan, prepare_noise_std_for_risk,
    limit_poisson_group_variance_planes, compute_covariance_aware_group_risk_from_plan,
    invert_aggregation_risks): per case the volume (also the Wiener pilot),
    member positions, sigma, attenuation, the group risk (float64) and weight."""
    from bmnd import aggregationweights, poisson, transforms, utils, variance, wiener
    from bmnd.profiles import BM3DProfile, BM4DProfile
    from bmnd.enums import AggregationWeightScope

    rng = np.random.default_rng(4321)
    out = {}
    cases = [
        ("ht2d", BM3DProfile(), (8, 8), (4, 9, 16), 19),
        ("wi2d", BM3DProfile(), (8, 8), (3, 8, 32), 19),
        ("ht3d", BM4DProfile(), (4, 4, 4), (2, 5, 16), 7),
        ("wi3d", BM4DProfile(), (5, 5, 5), (4, 7, 32), 7),
    ]
    for tag, prof, block, sizes, radius in cases:
        stage = "ht" if tag.startswith("ht") else "wiener"
        tlist = getattr(prof, f"{stage}_transform")
        beta = float(getattr(prof, f"{stage}_kaiser_beta"))
        vol_shape = tuple(b + 2 * radius + 3 for b in block)
        vol = rng.poisson(rng.uniform(3.0, 40.0, size=vol_shape)).astype(np.float32)
        vmodel = variance.build_poisson_variance_model(vol, variance_floor=1e-10, scale=1.0, source_name="observation")
        counts = tuple(s - b + 1 for s, b in zip(vol_shape, block))
        w_patch = utils.kaiser_window_nd(block, beta=beta)
        for n in sizes:
            # members clustered around a centre, so that many patches overlap
            centre = np.array([c // 2 for c in counts])
            pos = set()
            while len(pos) < n:
                pos.add(tuple(int(v) for v in np.clip(centre + rng.integers(-3, 4, size=len(block)), 0,
                                                       np.array(counts) - 1)))
            abs_pos = np.array(sorted(pos), dtype=np.int64)
            rng.shuffle(abs_pos)
            shifted = abs_pos - abs_pos.min(axis=0, keepdims=True)
            group_shape = (n,) + block
            fwd, inv = transforms.get_transform_matrix(group_shape, tlist)
            patches = np.stack([vol[tuple(slice(a, a + b) for a, b in zip(p, block))] for p in abs_pos])
            vpatches = np.stack([vmodel.variance_volume[tuple(slice(a, a + b) for a, b in zip(p, block))]
                                 for p in abs_pos])
            coef = transforms.apply_transform_nd(patches, fwd)
            for k in (1, 4):
                plan_ = variance.build_exact_poisson_group_plan(vmodel, abs_pos, shifted, group_shape, fwd)
                exact = plan_.prepare_noise_std_for_risk(k)
                if k >= n:
                    sigma = exact
                else:
                    approx = variance.get_direct_poisson_noise_std(vpatches, fwd, k=0)
                    sigma = variance.limit_poisson_group_variance_planes(exact, approx, k)
                if stage == "ht":
                    att = np.asarray(poisson._poisson_hard_threshold_mask(np.abs(coef), np.float32(3.0) * sigma, 1.0),
                                     dtype=np.float32)
                    risk = wiener.compute_covariance_aware_group_risk_from_plan(
                        att, plan_, inv, w_patch, exact_plane_count=k, noise_sigma=sigma)
                else:
                    att = wiener.compute_poisson_wiener_gain(coef, sigma, 0.4, eps=1e-10)
                    spow = wiener.compute_poisson_wiener_signal_power(coef, sigma, 0.4)
                    risk = wiener.compute_covariance_aware_group_risk_from_plan(
                        att, plan_, inv, w_patch, exact_plane_count=k, noise_sigma=sigma, signal_power=spow)
                weights = aggregationweights.invert_aggregation_risks(risk, group_size=n,
                                                                      scope=AggregationWeightScope.GROUP, eps=1e-10)
                key = f"{tag}_n{n}_k{k}"
                out[key + "_vol"] = vol
                out[key + "_abs"] = abs_pos
                out[key + "_sigma"] = np.asarray(sigma, dtype=np.float32)
                out[key + "_att"] = np.asarray(att, dtype=np.float32)
                out[key + "_risk"] = np.float64(risk)
                out[key + "_weights"] = np.asarray(weights, dtype=np.float32)
    path = os.path.join(HERE, "exact_risk_groups.npz")
    np.savez_compressed(path, **out)
    print(f"exact risk fixtures -> {path} ({len(out)} arrays)")


# Poisson cases with non-default profile fields: name -> (kind, generator, kwargs, profile fields)
OPTION_CASES = {
    "mass_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=21), dict(poisson_group_mass_conservation="both")),
    "mass_ht_bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=22),
                           dict(poisson_group_mass_conservation="ht")),
    "mass_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=23),
                           dict(poisson_group_mass_conservation="both")),
    "gain_classic_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=24),
                             dict(poisson_wiener_gain_mode="classic")),
    "gain_floor_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=25),
                                 dict(poisson_wiener_gain_mode="noise-floor")),
    "obs_variance_bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=26),
                                dict(poisson_variance_source_wiener="observation")),
    "obs_match_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=27),
                          dict(poisson_wiener_match_source="observation")),
    "soft_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=28), dict(ht_use_soft_thresholding=True)),
    "policy_finite_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=29),
                              dict(poisson_ht_match_policy="reference_finite_count")),
    "policy_std_bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=30),
                              dict(poisson_ht_match_policy="candidate_standardized")),
    "policy_finite_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=31),
                                    dict(poisson_ht_match_policy="reference_finite_count")),
    "risk_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=32), dict(wiener_weight_model="risk")),
    "group_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=33),
                      dict(ht_weight_scope="group", wiener_weight_scope="group")),
    "group_windowed_k0_bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=34),
                                     dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                                          wiener_weight_scope="group", wiener_weight_domain="windowed_synthesis",
                                          k=0)),
    "risk_windowed_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=35),
                                    dict(wiener_weight_model="risk", wiener_weight_domain="windowed_synthesis")),
    "exact_group_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=38),
                            dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                                 wiener_weight_scope="group", wiener_weight_domain="windowed_synthesis")),
    "exact_group_risk_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=39),
                                       dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                                            wiener_weight_model="risk", wiener_weight_scope="group",
                                            wiener_weight_domain="windowed_synthesis")),
    "exact_group_mass_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=41),
                                 dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                                      poisson_group_mass_conservation="both")),
    "exact_group_risk_bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=40),
                                    dict(wiener_weight_model="risk", wiener_weight_scope="group",
                                         wiener_weight_domain="windowed_synthesis", k=2)),
    "ssd_gamma_bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=36), dict(blockmatch_distance="ssd")),
    "ssd_gamma_bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=37),
                                dict(blockmatch_distance="ssd", gamma=2.5)),
}


def run_option(name: str) -> None:
    """opt_<case>.npz: like pipe_<case>.npz for a Poisson profile with the
    listed fields changed (stored as ``extra_json``)."""
    import json

    import bmnd as ref

    kind, gen, kwargs, extra = OPTION_CASES[name]
    clean, noisy = _make_input(gen, kwargs)
    profile_cls = ref.BM3DProfile if kind == "bm3d" else ref.BM4DProfile
    profile = profile_cls(noise_model=ref.NoiseModel.POISSON, **extra)
    stages, matches = {}, {}

    def stage_cb(stage, est):
        stages[stage] = np.asarray(est, dtype=np.float32)

    def bm_cb(stage, result):
        max_stack = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        matches[stage] = _pack_matches(result, max_stack, noisy.ndim)

    t0 = time.time()
    out = ref.bmnd(noisy, profile, stage_callback=stage_cb, blockmatch_callback=bm_cb)
    elapsed = time.time() - t0
    payload = dict(kind=np.array(kind), extra_json=np.array(json.dumps(extra)), clean=clean, noisy=noisy,
                   ht=stages["ht"], wiener=stages["wiener"], out=np.asarray(out, dtype=np.float32),
                   seconds=np.float64(elapsed))
    for stage, (sel, counts, accepted, refs) in matches.items():
        payload[f"{stage}_sel"] = sel
        payload[f"{stage}_count"] = counts
        payload[f"{stage}_accepted"] = accepted
        payload[f"{stage}_refs"] = refs
    path = os.path.join(HERE, f"opt_{name}.npz")
    np.savez_compressed(path, **payload)
    print(f"option {name}: {noisy.shape} in {elapsed:.1f} s -> {path}")


# Gaussian cases: name -> (profile kind, clean generator, kwargs, sigma, call options, profile fields)
GAUSS_CASES = {
    "bm3d_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=11), 3.0, {}, {}),
    "bm3d_40x24": ("bm3d", "ragged2d", dict(shape=(40, 24), seed=12), 2.0, {}, {}),
    "bm3d_est_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=13), 4.0, dict(estimate=True), {}),
    "bm3d_psd_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=14), 2.5, dict(psd=True), {}),
    "bm3d_conv_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=15), 3.0, {}, dict(nf=0)),
    "bm4d_12x16x20": ("bm4d", "ragged3d", dict(shape=(12, 16, 20), seed=16), 1.5, {}, {}),
    "bm3d_soft_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=17), 3.0, {}, dict(ht_use_soft_thresholding=True)),
    "bm3d_exact_group_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=18), 3.0, {},
                            dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                                 wiener_weight_model="risk", wiener_weight_scope="group",
                                 wiener_weight_domain="windowed_synthesis")),
    "bm3d_psd_group_32": ("bm3d", phantoms.shapes_2d, dict(size=32, seed=19), 2.5, dict(psd=True),
                          dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis",
                               wiener_weight_scope="group", wiener_weight_domain="windowed_synthesis")),
}


def _gauss_input(gen, kwargs, sigma):
    if gen in ("ragged2d", "ragged3d"):
        clean, _ = _make_input(gen, kwargs)
    else:
        clean, _ = gen(**kwargs)
    rng = np.random.default_rng(1000 + kwargs["seed"])
    noisy = (clean + sigma * rng.standard_normal(clean.shape)).astype(np.float32)
    return clean.astype(np.float32), noisy


def _colored_psd(shape, sigma):
    """A smooth, strictly positive PSD of mean N sigma^2 (low frequencies stronger)."""
    grids = np.meshgrid(*[np.fft.fftfreq(n) for n in shape], indexing="ij")
    r2 = sum(g * g for g in grids)
    psd = 1.0 + 3.0 * np.exp(-r2 / 0.02)
    psd *= float(np.prod(shape)) * sigma * sigma / psd.mean()
    return psd.astype(np.float32)


def run_gauss(name: str) -> None:
    """gauss_<case>.npz: the reference on stationary Gaussian noise (both stage
    estimates, both match sets, the sigma maps and the noise model's tables)."""
    import json

    import bmnd as ref
    from bmnd import variance as refvar

    kind, gen, kwargs, sigma, opts, extra = GAUSS_CASES[name]
    clean, noisy = _gauss_input(gen, kwargs, sigma)
    profile_cls = ref.BM3DProfile if kind == "bm3d" else ref.BM4DProfile
    profile = profile_cls(**extra)
    call = {}
    psd = None
    if opts.get("psd"):
        psd = _colored_psd(noisy.shape, sigma)
        call["sigma_psd"] = psd
    elif not opts.get("estimate"):
        call["sigma"] = sigma
    stages, matches = {}, {}

    def stage_cb(stage, est):
        stages[stage] = np.asarray(est, dtype=np.float32)

    def bm_cb(stage, result):
        max_stack = profile.ht_max_stack_size if stage == "ht" else profile.wiener_max_stack_size
        matches[stage] = _pack_matches(result, max_stack, noisy.ndim)

    t0 = time.time()
    out, smap = ref.bmnd(noisy, profile, return_sigma_map=True, stage_callback=stage_cb,
                         blockmatch_callback=bm_cb, **call)
    elapsed = time.time() - t0
    payload = dict(kind=np.array(kind), clean=clean, noisy=noisy, ht=stages["ht"], wiener=stages["wiener"],
                   out=np.asarray(out, dtype=np.float32), global_sigma=np.float64(smap["global"]),
                   sigma_ht=np.asarray(smap["ht"], dtype=np.float32),
                   sigma_wiener=np.asarray(smap["wiener"], dtype=np.float32), seconds=np.float64(elapsed),
                   sigma=np.float64(-1.0 if "sigma" not in call else sigma),
                   nf=np.array(-1 if "nf" not in extra else extra["nf"]),
                   soft=np.array(int(bool(extra.get("ht_use_soft_thresholding", False)))),
                   extra_json=np.array(json.dumps(extra)))
    if psd is not None:
        payload["sigma_psd"] = psd
    for stage, (sel, counts, accepted, refs) in matches.items():
        payload[f"{stage}_sel"] = sel
        payload[f"{stage}_count"] = counts
        payload[f"{stage}_accepted"] = accepted
        payload[f"{stage}_refs"] = refs
    # the noise model's tables, for the host-side restatement
    from bmnd.profilevalidation import resolve_profile as ref_resolve

    res = ref_resolve(profile, tuple(noisy.shape))
    model = refvar.build_variance_model(noisy, sigma=call.get("sigma"), sigma_psd=call.get("sigma_psd"),
                                       nf=res.effective_nf)
    payload["model_global_sigma"] = np.float64(model.global_sigma)
    payload["model_domain"] = np.array(model.variance_domain_shape, dtype=np.int64)
    from bmnd.transforms import get_transform_matrix

    for stage in ("ht", "wiener"):
        block = tuple(getattr(profile, f"{stage}_block_size"))
        fwd, _ = get_transform_matrix((2,) + block, getattr(profile, f"{stage}_transform"))
        payload[f"{stage}_cov_maps"] = np.asarray(
            refvar._get_cached_transformed_patch_cross_covariance(model, block, list(fwd[1:])), dtype=np.float32)
    payload["ht_noise_ssd"] = np.asarray(
        refvar.get_gaussian_blockmatch_noise_ssd(model, tuple(profile.ht_block_size),
                                                 tuple(profile.ht_search_window)), dtype=np.float32)
    path = os.path.join(HERE, f"gauss_{name}.npz")
    np.savez_compressed(path, **payload)
    print(f"gauss {name}: {noisy.shape} in {elapsed:.1f} s -> {path}")


def main(argv: list[str]) -> None:
    if not argv or argv[0] == "list":
        print("\n".join(PIPELINE_CASES))
        return
    if argv[0] == "unit":
        run_unit()
        return
    if argv[0] == "exact_risk":
        run_exact_risk()
        return
    if argv[0] == "sigma":
        for name in argv[1:]:
            run_sigma(name)
        return
    if argv[0] == "option":
        for name in argv[1:] or list(OPTION_CASES):
            run_option(name)
        return
    if argv[0] == "gauss":
        for name in argv[1:] or list(GAUSS_CASES):
            run_gauss(name)
        return
    if argv[0] == "pipeline":
        for name in argv[1:]:
            run_pipeline(name)
        return
    raise SystemExit(f"unknown command {argv[0]!r}")


if __name__ == "__main__":
    main(sys.argv[1:])
