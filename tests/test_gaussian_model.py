"""Host-side Gaussian noise model vs the reference's own tables (CPU only).

The fixtures ``tests/golden/gauss_*.npz`` hold, for each case, the
reference's global sigma, lag domain, covariance maps of both stages'
transformed patches and the SSD noise bias of the HT search window
(``tests/golden/make_golden.py gauss``)."""

import glob
import os

import numpy as np
import pytest

import bmnd_gb300 as bg
from bmnd_gb300 import gaussian, plan
from bmnd_gb300.validation import resolve_profile

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "gauss_*.npz")))


def _profile(g):
    kind = str(g["kind"])
    nf = int(g["nf"])
    extra = {} if nf < 0 else dict(nf=nf)
    if "soft" in g.files and int(g["soft"]):
        extra["ht_use_soft_thresholding"] = True
    return (bg.BM3DProfile if kind == "bm3d" else bg.BM4DProfile)(**extra)


def _model(g, profile):
    noisy = g["noisy"]
    sigma = float(g["sigma"])
    kw = {}
    if "sigma_psd" in g.files:
        kw["sigma_psd"] = g["sigma_psd"]
    elif sigma >= 0:
        kw["sigma"] = sigma
    res = resolve_profile(profile, noisy.shape)
    return gaussian.build_model(noisy.shape, profile.nf, volume=noisy, **kw), res


@pytest.mark.parametrize("case", CASES)
def test_model_tables_match_reference(case):
    g = np.load(os.path.join(GOLDEN, f"gauss_{case}.npz"))
    profile = _profile(g)
    model, res = _model(g, profile)
    assert model.domain == tuple(int(x) for x in g["model_domain"])
    assert model.global_sigma == pytest.approx(float(g["model_global_sigma"]), rel=1e-6)
    for stage in ("ht", "wiener"):
        block = tuple(int(b) for b in getattr(profile, f"{stage}_block_size"))
        maps = gaussian.covariance_maps(model, block, plan.spatial_forward(profile, g["noisy"].ndim, stage))
        want = g[f"{stage}_cov_maps"]
        assert maps.shape == want.shape
        scale = float(np.max(np.abs(want)))
        np.testing.assert_allclose(maps, want, rtol=0, atol=2e-6 * scale)
    ssd = gaussian.blockmatch_noise_ssd(model, tuple(profile.ht_block_size), tuple(profile.ht_search_window))
    np.testing.assert_allclose(ssd, g["ht_noise_ssd"], rtol=2e-6, atol=1e-6 * float(np.max(g["ht_noise_ssd"])))


def test_resolve_nf_rules():
    assert gaussian.resolve_nf(None, (10, 20)) == (None, False)
    assert gaussian.resolve_nf((), (10, 20)) == (None, False)
    assert gaussian.resolve_nf(0, (10, 40)) == ((10, 16), True)
    assert gaussian.resolve_nf((8, 0), (10, 40)) == ((10, 16), True)
    assert gaussian.resolve_nf((8, 12), (10, 40)) == ((8, 12), False)
    for bad in (True, 3, (1,), (1.5, 2), (-1, 2)):
        with pytest.raises(ValueError):
            gaussian.resolve_nf(bad, (10, 40))


def test_global_sigma_estimate_fallbacks():
    rng = np.random.default_rng(0)
    x = rng.normal(0, 2.0, size=20000).astype(np.float32)
    assert gaussian.estimate_global_sigma(x) == pytest.approx(2.0, rel=0.05)
    # MAD zero (most values equal) -> IQR, then the trimmed deviation, then sqrt(eps)
    y = np.full(100, 5.0, dtype=np.float32)
    y[:30] = np.linspace(0.1, 1.0, 30)
    assert gaussian.estimate_global_sigma(y) > 0
    assert gaussian.estimate_global_sigma(np.zeros(10, dtype=np.float32)) == pytest.approx(1e-5)


def test_white_noise_covariance_is_basis_autocorrelation():
    """For a scalar sigma the map of an orthonormal basis vector is sigma^2 at
    lag 0 and its (periodic) autocorrelation elsewhere."""
    model = gaussian.build_model((32, 32), (32, 32), sigma=2.0)
    prof = bg.BM3DProfile()
    maps = gaussian.covariance_maps(model, (8, 8), plan.spatial_forward(prof, 2, "wiener"))
    np.testing.assert_allclose(maps[:, 0, 0], 4.0, rtol=1e-5)
    # lags beyond the patch extent (and their periodic images) carry no covariance
    assert np.max(np.abs(maps[:, 8:25, :])) < 1e-4
