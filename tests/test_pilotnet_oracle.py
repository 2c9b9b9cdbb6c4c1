"""The pilot-net oracle itself (CPU): backward pass vs finite differences,
BF16 rounding, and the Poisson-deviance table used by the residual check."""

import numpy as np
import pytest

from oracle import pilotnet_ref as R


@pytest.mark.parametrize("ndim,shape", [(2, (2, 7, 9)), (3, (1, 5, 6, 7))])
def test_oracle_gradient_matches_finite_differences(ndim, shape):
    rng = np.random.default_rng(0)
    C, L = 8, 4
    p = R.init_params(ndim, C, L, seed=1, out_scale=1.0).astype(np.float64)
    x = rng.poisson(5.0, size=shape).astype(np.float64)
    t = 0.8 * x + 1.0
    _, g, _ = R.loss_and_gradient(p, x, t, ndim, C, L, bf16=False)
    idx = rng.choice(p.size, 30, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        lp = R.loss_and_gradient(p + e, x, t, ndim, C, L, bf16=False)[0]
        lm = R.loss_and_gradient(p - e, x, t, ndim, C, L, bf16=False)[0]
        num = (lp - lm) / 2e-6
        assert abs(num - g[i]) <= 1e-5 * max(abs(num), 1e-3), (i, num, g[i])


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(0, 10, 20000), rng.normal(0, 1e-3, 2000), [0.0, -0.0, 1.0, 65504.0]])
    x = x.astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(R.bf16_round(x), want)


def test_deviance_table_limits():
    from bmnd_gb300.pilot import deviance_table

    mus, ev, vv = deviance_table(n=64)
    # large mean: E ~ 1 + 1/(6 mu), Var ~ 2
    big = mus > 200
    assert np.all(np.abs(ev[big] - (1.0 + 1.0 / (6.0 * mus[big]))) < 5e-3)
    assert np.all(np.abs(vv[big] - 2.0) < 0.05)
    # small mean: E ~ 2 mu ln(1/mu) dominated, and always below its large-mean value
    assert np.all(ev[mus < 0.01] < 0.2)
    assert np.all(np.diff(ev[mus < 1.0]) > 0)
