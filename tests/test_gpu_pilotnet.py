"""Learned pilot on the GPU: kernels vs the CPU oracle (forward, gradients),
the residual check, training, and the fast path's fallback."""

import numpy as np
import pytest

from oracle import pilotnet_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["tcgen05", "mma_sync"])
def engine(request, native):
    from bmnd_gb300.pilot import get_conv_engine, set_conv_engine

    old = get_conv_engine()
    set_conv_engine(request.param)
    yield request.param
    set_conv_engine(old)


def _net(cuda, ndim, channels, layers, seed):
    from bmnd_gb300.pilot import PilotNet

    params = R.init_params(ndim, channels, layers, seed=seed, out_scale=1.0)
    return PilotNet(ndim, channels, layers, params=params), params


@pytest.mark.parametrize("ndim,channels,layers,shape", [
    (3, 48, 4, (2, 10, 12, 20)),
    (3, 32, 3, (1, 9, 17, 18)),
    (2, 32, 4, (2, 20, 36)),
    (2, 48, 5, (1, 33, 17)),
    (3, 48, 3, (3, 1, 19, 9)),   # one-plane volumes in a batch: both z-halo planes belong to neighbours
])
def test_forward_and_gradient_match_oracle(cuda, engine, ndim, channels, layers, shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.poisson(rng.uniform(1, 30, size=shape)).astype(np.float32)
    t = (0.7 * x + 2.0).astype(np.float32)
    net, params = _net(cuda, ndim, channels, layers, seed=7)
    xg = cuda.from_numpy(x).cuda()
    tg = cuda.from_numpy(t).cuda()
    # forward (inference path, ping-pong activations) vs the oracle's BF16 mirror
    pilot_g, y_g = net.forward(xg, want_y=True)
    net.check_status()
    pilot_o, y_o, _ = R.forward(params, x, ndim, channels, layers, bf16=True)
    y_g = y_g.cpu().numpy()
    assert np.max(np.abs(y_g - y_o)) <= 2e-2 * max(1.0, np.max(np.abs(y_o))), np.max(np.abs(y_g - y_o))
    assert np.corrcoef(y_g.ravel(), y_o.ravel())[0, 1] > 0.9999
    # gradient pass (keeps every activation) vs the oracle
    loss_g, grad_g = net.gradient(xg, tg)
    net.check_status(training=True)
    loss_o, grad_o, _ = R.loss_and_gradient(params, x, t, ndim, channels, layers, bf16=True)
    assert abs(float(loss_g.item()) - loss_o) <= 1e-3 * loss_o + 1e-7
    grad_g = grad_g.cpu().numpy().astype(np.float64)
    off = 0
    for l, (taps, cin, cout) in enumerate(R.layer_shapes(ndim, channels, layers)):
        n = taps * cin * cout + cout
        a, b = grad_g[off:off + n], grad_o[off:off + n]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert rel < 3e-2, (l, rel)
        off += n


@pytest.mark.parametrize("ndim,channels,layers,shape", [
    (3, 48, 6, (2, 40, 70, 66)),    # thousands of tiles per launch, ragged x and y edges
    (2, 32, 5, (3, 300, 129)),
])
def test_tensor_memory_engine_matches_warp_mma(cuda, native, ndim, channels, layers, shape):
    """The tcgen05 layers (persistent CTAs, double-buffered halo tiles) against
    the mma.sync layers on volumes too large for the oracle: same BF16 inputs,
    FP32 accumulation in a different order."""
    from bmnd_gb300.pilot import get_conv_engine, set_conv_engine

    rng = np.random.default_rng(3)
    x = rng.poisson(rng.uniform(1, 30, size=shape)).astype(np.float32)
    t = (0.7 * x + 2.0).astype(np.float32)
    net, _ = _net(cuda, ndim, channels, layers, seed=4)
    xg, tg = cuda.from_numpy(x).cuda(), cuda.from_numpy(t).cuda()
    old = get_conv_engine()
    res = {}
    try:
        for eng in ("mma_sync", "tcgen05"):
            set_conv_engine(eng)
            _, y = net.forward(xg, want_y=True)
            net.check_status()
            loss, grad = net.gradient(xg, tg)
            net.check_status(training=True)
            res[eng] = (y.cpu().numpy(), float(loss.item()), grad.cpu().numpy().astype(np.float64))
    finally:
        set_conv_engine(old)
    (ya, la, ga), (yb, lb, gb) = res["mma_sync"], res["tcgen05"]
    scale = max(1.0, float(np.max(np.abs(ya))))
    assert np.max(np.abs(ya - yb)) <= 2e-2 * scale, np.max(np.abs(ya - yb))
    assert np.corrcoef(ya.ravel(), yb.ravel())[0, 1] > 0.99999
    assert abs(la - lb) <= 1e-3 * abs(la) + 1e-7
    assert np.linalg.norm(ga - gb) / np.linalg.norm(ga) < 2e-2


def test_tensor_core_wait_runs_out_and_recovers(cuda, native):
    """Failure detection without a GPU fault: with the wait probe set, every
    tcgen05 layer waits 2 ms on an mbarrier that nothing completes, in the
    forward and in the gradient pass; the wait runs out, the launches stop with
    their tensor memory freed, and the status call reports BMND_ERR_TIMEOUT.
    The next forward and gradient passes (probe off) run and equal the ones
    before the probe bit for bit, which also shows that the tensor memory was
    given back (an allocation would wait otherwise)."""
    from bmnd_gb300 import _abi
    from bmnd_gb300.pilot import get_conv_engine, set_conv_engine

    rng = np.random.default_rng(11)
    x = cuda.from_numpy(rng.poisson(rng.uniform(1, 20, size=(1, 20, 36, 40))).astype(np.float32)).cuda()
    t = 0.7 * x + 2.0
    net, _ = _net(cuda, 3, 48, 5, seed=12)
    lib = _abi.lib()
    old = get_conv_engine()
    try:
        set_conv_engine("tcgen05")
        before = net.forward(x).clone()
        net.check_status()
        _, grad_before = net.gradient(x, t)
        grad_before = grad_before.clone()
        net.check_status(training=True)
        _abi.check(lib.bmnd_pilotnet_set_wait_probe(2_000_000))
        try:
            net.forward(x)
            with pytest.raises(_abi.BmndError) as info:
                net.check_status()
            assert info.value.code == _abi.ERR_TIMEOUT
            # the gradient pass: the tensor-core layers and weight gradients
            # (512 tensor-memory columns each) time out the same way
            net.gradient(x, t)
            with pytest.raises(_abi.BmndError) as info:
                net.check_status(training=True)
            assert info.value.code == _abi.ERR_TIMEOUT
        finally:
            _abi.check(lib.bmnd_pilotnet_set_wait_probe(0))
        after = net.forward(x)
        net.check_status()
        assert cuda.equal(after, before)
        _, grad_after = net.gradient(x, t)
        net.check_status(training=True)
        assert cuda.equal(grad_after, grad_before)
    finally:
        set_conv_engine(old)
    with pytest.raises(_abi.BmndError):
        _abi.check(lib.bmnd_pilotnet_set_wait_probe(2_000_000_000))


def test_tile_deviance_matches_numpy(cuda, native):
    from bmnd_gb300.pilot import deviance_table, tile_zscores

    rng = np.random.default_rng(11)
    mu = rng.uniform(0.5, 40.0, size=(20, 24, 37)).astype(np.float32)
    x = rng.poisson(mu).astype(np.float32)
    z, grid = tile_zscores(cuda.from_numpy(x).cuda(), cuda.from_numpy(mu).cuda(), 8)
    assert grid == (3, 3, 5)
    mus, ev, vv = deviance_table()
    lm = np.log(mus)
    e = np.interp(np.log(mu), lm, ev)
    v = np.interp(np.log(mu), lm, vv)
    with np.errstate(divide="ignore", invalid="ignore"):
        d = 2 * (np.where(x > 0, x * np.log(np.where(x > 0, x, 1) / mu), 0) - (x - mu))
    for (i, j, k) in [(0, 0, 0), (2, 1, 4), (1, 2, 3)]:
        sl = (slice(8 * i, 8 * i + 8), slice(8 * j, 8 * j + 8), slice(8 * k, 8 * k + 8))
        zz = (d[sl].sum() - e[sl].sum()) / np.sqrt(v[sl].sum())
        assert abs(z[i, j, k] - zz) < 1e-2 * max(1.0, abs(zz)), (i, j, k, z[i, j, k], zz)
    # the true mean gives unremarkable scores, a wrong mean does not
    assert np.all(np.abs(z) < 6)
    z2, _ = tile_zscores(cuda.from_numpy(x).cuda(), cuda.from_numpy(0.5 * mu).cuda(), 8)
    assert np.all(z2 > 6)


def test_training_reduces_loss(cuda, native):
    from bmnd_gb300.pilot import PilotNet

    rng = np.random.default_rng(5)
    pairs = []
    for _ in range(2):
        mu = np.full((24, 24, 24), 10.0, dtype=np.float32)
        mu[6:18, 4:20, 8:16] = 25.0
        x = rng.poisson(mu).astype(np.float32)
        pairs.append((cuda.from_numpy(x).cuda(), cuda.from_numpy(mu).cuda()))
    net = PilotNet(3, 32, 4, seed=0)
    hist = net.fit(pairs, steps=200, crop=16, batch=2, lr=3e-4, log_every=20)
    assert hist[-1][1] < 0.8 * hist[0][1], hist


def test_fallback_replaces_failing_tiles(cuda, native):
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.api import stage_device
    from bmnd_gb300.pilot import PilotNet, bmnd_fast

    clean, noisy = phantoms.ellipsoids_3d(40, seed=3)
    x = cuda.from_numpy(noisy).cuda()
    profile = bg.BM4DProfile(noise_model=bg.NoiseModel.POISSON)
    # an untrained net with a large residual branch: the check must reject it
    net = PilotNet(3, 32, 3, params=R.init_params(3, 32, 3, seed=2, out_scale=30.0))
    d = {}
    out = bmnd_fast(x, profile, net, tile=16, excess_high=0.5, details=d)
    assert d["fallback_tiles"] == d["tiles"]
    # every tile was recomputed by plain stage 1 (on the tile plus its halo)
    plain_pilot = stage_device(x, profile, "ht").cpu().numpy()
    fb = d["pilot"].cpu().numpy()
    assert abs(phantoms.psnr(fb, clean) - phantoms.psnr(plain_pilot, clean)) < 0.3
    assert bool(cuda.isfinite(out).all())


def test_mma_rates_measured(cuda, native):
    """bmnd_mma_rates: clocks per 128 x N x 16 BF16 MMA on every SM, finite and
    ordered as the operand reads predict (a wider N never costs less)."""
    from bmnd_gb300 import _abi

    r = _abi.mma_rates(((48, 2), (128, 2), (256, 2), (48, 1)))
    clk = [c for _, _, c in r]
    assert all(10.0 < c < 2000.0 for c in clk), r
    assert clk[0] <= 1.05 * clk[1] and clk[1] <= 1.05 * clk[2], r
