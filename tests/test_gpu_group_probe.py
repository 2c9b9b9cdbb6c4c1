"""The group filter kernel, group by group, against the reference.

``bmnd_group_probe`` runs the filter on explicit groups and returns each
group's intermediate arrays, so the hardest kernel of the path (the exact
overlap-aware noise variance) is checked on its own, not only through whole
images:

* the reference's per-group fixtures (``tests/golden/unit_reference.npz``,
  ``grp_*``: hard-thresholding and Wiener transforms, 2-D and 3-D, n = 1 ... 32
  members on a Poisson(20) volume, made by the reference's own
  get_direct_poisson_noise_std, _poisson_hard_threshold_mask,
  compute_aggregation_weights and compute_poisson_wiener_gain): forward
  coefficients, exact and approximate sigma, hard-threshold mask (decisions
  within 1e-5 of their threshold excepted), weights, filtered patches and
  Wiener gain;
* the exact sigma against the diagonal of the dense covariance
  diag(E Cov E^T), E = kron(G, S) (as tests/test_variance_unit.py:747-779 of the
  reference does), in float64 NumPy;
* the reference's small 1-D cases: exact equals the dense diagonal with k = n
  and k > n, exact equals approximate without overlap
  (test_variance_unit.py:719-744, :747-779);
* the plane limiting rule (variance.py:1572-1631, test_variance_unit.py:496-513):
  the first k planes exact, the others rescaled so that each coefficient's
  total over the planes is the approximate total.
"""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [f"{tag}_n{n}" for tag, ns in (("ht2d", (1, 2, 4, 8, 16)), ("wi2d", (1, 2, 4, 8, 32)),
                                         ("ht3d", (1, 2, 4, 8, 16)), ("wi3d", (1, 2, 4, 8, 32)))
         for n in ns]


def _params(tag, shape, k=4, filt="ht"):
    import bmnd_gb300 as bg
    from bmnd_gb300 import _abi, plan
    from bmnd_gb300.enums import BlockMatchDistance

    prof = (bg.BM3DProfile if tag.endswith("2d") else bg.BM4DProfile)(noise_model=bg.NoiseModel.POISSON)
    p = plan.stage_params(prof, shape, "ht" if tag.startswith("ht") else "wiener",
                          BlockMatchDistance.POISSON_DEVIANCE, k)
    p.filter = _abi.FILTER_HARD_THRESHOLD if filt == "ht" else _abi.FILTER_WIENER
    p.ht_lambda = 3.0
    p.wiener_scale = 0.4
    return p


def _probe(cuda, p, vol, sel, cnt, pilot=None):
    from bmnd_gb300.api import group_probe

    x = cuda.from_numpy(np.ascontiguousarray(vol, dtype=np.float32)).cuda()
    pt = None if pilot is None else cuda.from_numpy(np.ascontiguousarray(pilot, dtype=np.float32)).cuda()
    return group_probe(p, x, sel, cnt, pilot=pt)


def _ht_margin(coef, sigma, lam=3.0, scale=1.0):
    """Relative distance of each hard-threshold decision from its boundary
    (poisson.py:30-46), float64."""
    cc = np.abs(coef.astype(np.float64)) / scale
    tc = (np.float32(lam) * sigma.astype(np.float32)).astype(np.float64) / scale
    tol = 128.0 * 1.1920928955078125e-07 * np.maximum(np.maximum(cc, tc), 1.0)
    bound = tc + tol
    return np.abs(cc - bound) / np.maximum(bound, 1e-300)


def _case(g, key):
    vol = g[key + "_vol"]
    abs_pos = g[key + "_abs"]
    tag = key.split("_")[1]
    block = (8, 8) if tag.endswith("2d") else ((4, 4, 4) if tag == "ht3d" else (5, 5, 5))
    counts = tuple(s - b + 1 for s, b in zip(vol.shape, block))
    lins = np.ravel_multi_index(tuple(abs_pos.T), counts).astype(np.int32)
    return tag, vol, block, lins


@pytest.mark.parametrize("case", CASES)
def test_group_filter_matches_reference_fixture(cuda, native, case):
    g = np.load(os.path.join(GOLDEN, "unit_reference.npz"))
    key = f"grp_{case}"
    tag, vol, block, lins = _case(g, key)
    n = lins.size
    P = int(np.prod(block))
    p = _params(tag, vol.shape)
    sel = np.full((1, p.max_stack), -1, dtype=np.int32)
    sel[0, :n] = lins
    cnt = np.array([n], dtype=np.int32)
    res = _probe(cuda, p, vol, sel, cnt)
    coef = res["coef"][0, :n].reshape((n,) + block)
    sigma = res["sigma"][0, :n].reshape((n,) + block)
    mask = res["atten"][0, :n].reshape((n,) + block)
    ref_coef, ref_sigma = g[key + "_coef"], g[key + "_sigma"]

    # forward coefficients: the same float32 products (one FMA per term)
    scale_c = float(np.max(np.abs(ref_coef)))
    np.testing.assert_allclose(coef, ref_coef, rtol=1e-6, atol=1e-6 * scale_c)
    # exact sigma of the first min(4, n) planes, then the plane limiting
    scale_s = float(np.max(ref_sigma))
    np.testing.assert_allclose(sigma, ref_sigma, rtol=2e-5, atol=2e-6 * scale_s)
    # approximate sigma (k = 0): squared transforms of the variance group
    res0 = _probe(cuda, _params(tag, vol.shape, k=0), vol, sel, cnt)
    sig0 = res0["sigma"][0, :n].reshape((n,) + block)
    np.testing.assert_allclose(sig0, g[key + "_sigma_approx"], rtol=2e-5, atol=2e-6 * scale_s)
    # hard-threshold mask: identical wherever the decision is not within 1e-5 of its threshold
    ref_mask = g[key + "_mask"].astype(np.float32)
    decided = _ht_margin(ref_coef, ref_sigma) > 1e-5
    assert np.array_equal(mask[decided], ref_mask[decided])
    # weights and filtered patches (float32 plane risks here, float64 in the reference)
    np.testing.assert_allclose(res["weights"][0, :n], g[key + "_weights_ht"], rtol=1e-4)
    if np.array_equal(mask, ref_mask):
        filt = res["filt"][0, :n].reshape((n,) + block)
        ref_filt = g[key + "_filt_ht"]
        np.testing.assert_allclose(filt, ref_filt, rtol=1e-5, atol=1e-5 * float(np.max(np.abs(ref_filt))))
    # Wiener gain with the observation as its own pilot: gain(coef, sigma, mu^2 = 0.4)
    resw = _probe(cuda, _params(tag, vol.shape, filt="wiener"), vol, sel, cnt, pilot=vol)
    gain = resw["atten"][0, :n].reshape((n,) + block)
    np.testing.assert_allclose(gain, g[key + "_gain"], atol=2e-5)
    assert P == res["coef"].shape[2]


def _dense_exact_variance(vol, block, abs_pos, G, spatial, k):
    """diag(E Cov E^T) for the first k planes in float64: E = kron(G[:k], S),
    Cov the covariance of the stacked patch entries (V at a shared voxel, else 0)."""
    S = np.ones((1, 1))
    for m in spatial:
        S = np.kron(S, np.asarray(m, dtype=np.float64))
    n = abs_pos.shape[0]
    P = int(np.prod(block))
    E = np.kron(np.asarray(G, dtype=np.float64)[:k], S)  # (k P) x (n P)
    offs = np.stack(np.unravel_index(np.arange(P), block), axis=1)
    vox = np.ravel_multi_index(tuple((abs_pos[:, None, :] + offs[None]).reshape(-1, len(block)).T), vol.shape)
    uniq, inv = np.unique(vox, return_inverse=True)
    A = np.zeros((uniq.size, n * P))
    A[inv, np.arange(n * P)] = 1.0
    V = np.maximum(vol.reshape(-1)[uniq].astype(np.float64), 1e-10)
    B = E @ A.T
    return (B * B) @ V


@pytest.mark.parametrize("case", ["ht2d_n16", "wi2d_n32", "ht3d_n8", "ht3d_n16", "wi3d_n32"])
def test_exact_sigma_equals_dense_covariance_diagonal(cuda, native, case):
    from bmnd_gb300 import transforms

    g = np.load(os.path.join(GOLDEN, "unit_reference.npz"))
    tag, vol, block, lins = _case(g, f"grp_{case}")
    abs_pos = g[f"grp_{case}_abs"]
    n = lins.size
    p = _params(tag, vol.shape, k=n)  # every plane exact
    sel = np.full((1, p.max_stack), -1, dtype=np.int32)
    sel[0, :n] = lins
    res = _probe(cuda, p, vol, sel, np.array([n], dtype=np.int32))
    sigma = res["sigma"][0, :n].astype(np.float64)
    G = transforms.haar_group_matrix(n)
    spatial = [np.array(p.spatial_fwd[a][: block[a] * block[a]], dtype=np.float32).reshape(block[a], block[a])
               for a in range(len(block))]
    dense = _dense_exact_variance(vol, block, abs_pos, G, spatial, n).reshape(n, -1)
    np.testing.assert_allclose(sigma ** 2, dense, rtol=2e-5, atol=1e-6 * float(dense.max()))


def _manual_params(shape, block, G_kind, spatial, k, filt="ht"):
    from bmnd_gb300 import _abi

    p = _abi.StageParams()
    p.ndim = len(shape)
    for a in range(len(shape)):
        p.shape[a], p.block[a], p.search_radius[a] = shape[a], block[a], 1
    p.max_stack, p.min_stack = 2, 1
    p.distance = _abi.DIST_POISSON_DEVIANCE
    p.stabilize_ties = 1
    p.filter = _abi.FILTER_HARD_THRESHOLD if filt == "ht" else _abi.FILTER_WIENER
    p.group_transform = G_kind
    p.variance_k = k
    p.weight_model = _abi.WEIGHT_VARIANCE
    p.match_threshold, p.ht_lambda, p.wiener_scale = 1.0, 3.0, 0.4
    p.count_scale, p.variance_floor, p.eps = 1.0, 1e-10, 1e-10
    p.noise_model = _abi.NOISE_POISSON
    for a, m in enumerate(spatial):
        m = np.asarray(m, dtype=np.float32)
        for i, v in enumerate(m.reshape(-1)):
            p.spatial_fwd[a][i] = float(v)
        for i, v in enumerate(m.T.reshape(-1)):
            p.spatial_inv[a][i] = float(v)
    for i in range(int(np.prod(block))):
        p.window[i] = 1.0
    return p


HAAR2 = (np.float32(1.0 / np.sqrt(2.0)) * np.array([[1.0, 1.0], [1.0, -1.0]])).astype(np.float32)


@pytest.mark.parametrize("k", [2, 3], ids=["full", "overfull"])
def test_exact_sigma_dense_diagonal_reference_case(cuda, native, k):
    """test_variance_unit.py:747-779: volume [1, 2, 5], overlapping patches at 0
    and 1 of length 2, Haar on both axes."""
    from bmnd_gb300 import _abi

    vol = np.array([1.0, 2.0, 5.0], dtype=np.float32)
    p = _manual_params((3,), (2,), _abi.GROUP_HAAR, [HAAR2], k)
    sel = np.array([[0, 1]], dtype=np.int32)
    res = _probe(cuda, p, vol, sel, np.array([2], dtype=np.int32))
    dense = _dense_exact_variance(vol, (2,), np.array([[0], [1]]), HAAR2, [HAAR2], 2)
    np.testing.assert_allclose(res["sigma"][0].reshape(-1).astype(np.float64) ** 2, dense, atol=1e-6)


def test_exact_sigma_equals_approximate_without_overlap(cuda, native):
    """test_variance_unit.py:719-744: patches at 0 and 2 do not overlap, so the
    exact and the approximate sigma agree."""
    from bmnd_gb300 import _abi

    vol = np.array([1.0, 2.0, 3.0, 4.0], dtype=np.float32)
    sel = np.array([[0, 2]], dtype=np.int32)
    cnt = np.array([2], dtype=np.int32)
    exact = _probe(cuda, _manual_params((4,), (2,), _abi.GROUP_HAAR, [HAAR2], 2), vol, sel, cnt)["sigma"]
    approx = _probe(cuda, _manual_params((4,), (2,), _abi.GROUP_HAAR, [HAAR2], 0), vol, sel, cnt)["sigma"]
    np.testing.assert_allclose(exact, approx, atol=1e-6)


@pytest.mark.parametrize("case", ["ht2d_n16", "wi3d_n32"])
def test_plane_limiting_keeps_the_approximate_total(cuda, native, case):
    """variance.py:1572-1631: with k = 1 the first plane is exact and the
    others are rescaled so that every coefficient's total over the planes is
    max(approximate total, exact first plane)."""
    g = np.load(os.path.join(GOLDEN, "unit_reference.npz"))
    tag, vol, block, lins = _case(g, f"grp_{case}")
    n = lins.size
    cnt = np.array([n], dtype=np.int32)

    def run(k):
        p = _params(tag, vol.shape, k=k)
        s = np.full((1, p.max_stack), -1, dtype=np.int32)
        s[0, :n] = lins
        return _probe(cuda, p, vol, s, cnt)["sigma"][0, :n].astype(np.float64)

    approx, one, full = run(0), run(1), run(n)
    np.testing.assert_allclose(one[0], full[0], rtol=1e-6)
    total = np.maximum((approx ** 2).sum(axis=0), full[0] ** 2)
    np.testing.assert_allclose((one ** 2).sum(axis=0), total, rtol=1e-5)


RISK_KEYS = [f"{tag}_n{n}_k{k}" for tag, ns in (("ht2d", (4, 9, 16)), ("wi2d", (3, 8, 32)), ("ht3d", (2, 5, 16)),
                                                ("wi3d", (4, 7, 32))) for n in ns for k in (1, 4)]


@pytest.mark.parametrize("key", RISK_KEYS)
def test_exact_risk_weight_matches_reference(cuda, native, key):
    """The covariance-aware exact group weighting on single groups against the
    reference's own compute_covariance_aware_group_risk_from_plan and
    invert_aggregation_risks (``exact_risk_groups.npz``, clustered members on
    a Poisson volume, k = 1 and 4): sigma, the attenuation (hard-threshold
    mask, or Wiener gain with the observation as its own pilot and the risk
    model's bias term) and the one weight of the group, 1 / (risk + eps)."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import plan
    from bmnd_gb300.enums import BlockMatchDistance
    from bmnd_gb300.validation import resolve_profile

    g = np.load(os.path.join(GOLDEN, "exact_risk_groups.npz"))
    tag = key.split("_")[0]
    vol, abs_pos = g[key + "_vol"], g[key + "_abs"]
    k = int(key.rsplit("_k", 1)[1])
    block = (8, 8) if tag.endswith("2d") else ((4, 4, 4) if tag == "ht3d" else (5, 5, 5))
    stage = "ht" if tag.startswith("ht") else "wiener"
    opts = dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis", wiener_weight_model="risk",
                wiener_weight_scope="group", wiener_weight_domain="windowed_synthesis")
    prof = (bg.BM3DProfile if tag.endswith("2d") else bg.BM4DProfile)(noise_model=bg.NoiseModel.POISSON, **opts)
    resolve_profile(prof, vol.shape)  # the option strings become enums
    p = plan.stage_params(prof, vol.shape, stage, BlockMatchDistance.POISSON_DEVIANCE, k)
    assert p.exact_risk_weights == 1
    p.ht_lambda, p.wiener_scale = 3.0, 0.4
    counts = tuple(s - b + 1 for s, b in zip(vol.shape, block))
    lins = np.ravel_multi_index(tuple(abs_pos.T), counts).astype(np.int32)
    n = lins.size
    sel = np.full((1, p.max_stack), -1, dtype=np.int32)
    sel[0, :n] = lins
    res = _probe(cuda, p, vol, sel, np.array([n], dtype=np.int32), pilot=vol if stage == "wiener" else None)
    sigma = res["sigma"][0, :n].reshape((n,) + block)
    att = res["atten"][0, :n].reshape((n,) + block)
    ref_sigma, ref_att = g[key + "_sigma"], g[key + "_att"]
    np.testing.assert_allclose(sigma, ref_sigma, rtol=2e-5, atol=2e-6 * float(np.max(ref_sigma)))
    if stage == "ht" and not np.array_equal(att, ref_att):
        # a decision within float rounding of its threshold changes the risk: the rest must agree
        coef = res["coef"][0, :n].reshape((n,) + block)
        assert np.all(_ht_margin(coef, ref_sigma)[att != ref_att] <= 1e-5)
        pytest.skip("a hard-threshold decision sits on its threshold")
    np.testing.assert_allclose(att, ref_att, rtol=1e-5, atol=2e-6)
    w = res["weights"][0, :n]
    assert np.all(w == w[0])
    np.testing.assert_allclose(w, g[key + "_weights"], rtol=2e-5)
