"""What the trained pilot net gains (GPU), on a held-out phantom crop.

The committed weights (bmnd_gb300/weights/pilot_bm4d.npz) were trained by
``python -m bmnd_gb300.train_pilot`` on seeds 1000-1007; this test uses a
128^3 crop of the 256^3 phantom with seed 2001 (same structure scale)."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(cuda, native):
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.pilot import PilotNet, default_net_path

    path = default_net_path("bm4d")
    if not os.path.exists(path):
        pytest.skip("no trained weights")
    clean, noisy = phantoms.ellipsoids_3d(256, seed=2001)
    sl = (slice(64, 192),) * 3
    clean, noisy = np.ascontiguousarray(clean[sl]), np.ascontiguousarray(noisy[sl])
    x = cuda.from_numpy(noisy).cuda()
    prof = bg.BM4DProfile(noise_model=bg.NoiseModel.POISSON)
    return dict(clean=clean, noisy=noisy, x=x, prof=prof, net=PilotNet.load(path))


def test_trained_pilot_beats_untrained_and_no_pilot(cuda, case):
    from bmnd_gb300 import phantoms
    from bmnd_gb300.api import stage_device
    from bmnd_gb300.pilot import PilotNet, bmnd_fast, fast_profile

    clean, x, prof, net = case["clean"], case["x"], case["prof"], case["net"]
    trained = bmnd_fast(x, prof, net, check=False)
    untrained = bmnd_fast(x, prof, PilotNet(net.ndim, net.channels, net.layers, seed=0), check=False)
    no_pilot = stage_device(x, fast_profile(prof), "wiener", x, match_precision="approx")
    p_tr = phantoms.psnr(trained.cpu().numpy(), clean)
    p_un = phantoms.psnr(untrained.cpu().numpy(), clean)
    p_np = phantoms.psnr(no_pilot.cpu().numpy(), clean)
    assert p_tr > p_un + 3.0, (p_tr, p_un)
    assert p_tr > p_np + 3.0, (p_tr, p_np)


def test_trained_pilot_tracks_plain_stage1(cuda, case):
    from bmnd_gb300 import phantoms
    from bmnd_gb300.api import stage_device

    clean, x, prof, net = case["clean"], case["x"], case["prof"], case["net"]
    plain1 = stage_device(x, prof, "ht").cpu().numpy()
    learned = net.forward(x).cpu().numpy()
    # the net imitates plain stage 1: close to it, and far better than the input
    assert phantoms.psnr(learned, plain1) > 38.0
    assert phantoms.psnr(learned, clean) > phantoms.psnr(case["noisy"], clean) + 12.0


def test_fast_path_within_budget_of_plain_path(cuda, case):
    """The learned-pilot path keeps the plain path's quality (PSNR loss at most
    0.05 dB on the held-out crop) and beats the method without the net: plain
    stage 1 followed by the same fast Wiener stage."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.api import stage_device
    from bmnd_gb300.pilot import FAST_MATCH_PRECISION, bmnd_fast, fast_profile

    clean, x, prof, net = case["clean"], case["x"], case["prof"], case["net"]
    plain = bg.bmnd_device(x, prof).cpu().numpy()
    fast = bmnd_fast(x, prof, net).cpu().numpy()
    no_net = stage_device(x, fast_profile(prof), "wiener", stage_device(x, prof, "ht"),
                          match_precision=FAST_MATCH_PRECISION, fast_transforms=True).cpu().numpy()
    p_plain, p_fast, p_nonet = (phantoms.psnr(v, clean) for v in (plain, fast, no_net))
    print(f"held-out 128^3: plain {p_plain:.3f} dB, learned fast path {p_fast:.3f} dB, "
          f"plain stage 1 + fast stage 2 {p_nonet:.3f} dB")
    assert p_fast >= p_plain - 0.05, (p_fast, p_plain)
    assert p_fast > p_nonet, (p_fast, p_nonet)


def test_learned_pilot_through_bmnd(cuda, case):
    """bmnd(..., pilot="learned") is the fast path behind the drop-in API: NumPy
    in, NumPy out, the pilot reported as the "ht" stage estimate."""
    import bmnd_gb300 as bg
    from bmnd_gb300.pilot import bmnd_fast

    noisy, x, prof, net = case["noisy"], case["x"], case["prof"], case["net"]
    seen = {}
    out = bg.bmnd(noisy, prof, pilot="learned", stage_callback=lambda s, e: seen.__setitem__(s, e))
    assert isinstance(out, np.ndarray) and out.dtype == np.float32 and out.shape == noisy.shape
    details = {}
    ref = bmnd_fast(x, prof, net, details=details).cpu().numpy()
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-4 * float(np.max(ref)))
    np.testing.assert_array_equal(seen["wiener"], out)
    np.testing.assert_allclose(seen["ht"], details["pilot"].cpu().numpy(), rtol=0, atol=1e-4 * float(np.max(ref)))
    with pytest.raises(NotImplementedError):
        bg.bmnd(noisy, prof, pilot="learned", return_sigma_map=True)
    with pytest.raises(ValueError):
        bg.bmnd(noisy, prof, pilot="neural")


def test_lowcount_pilot_on_uneven_volume(cuda, native):
    """The low-count 3-D net (bmnd_gb300/weights/pilot_bm4d_lowcount.npz,
    trained on 400 volumes of 128^3 at peaks U[2, 5], seeds 3000-3399) on a
    held-out volume of uneven extents at a peak drawn from the same range:
    the fast path through bmnd() stays within 0.4 dB of the plain path (the
    eight 128^3-320^3 evaluation volumes range from -0.36 to +0.28 dB), far
    above the noisy input, and reports its tile fallback."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.pilot import PilotNet, bmnd_fast, default_net_path, lowcount_peak

    path = default_net_path("bm4d_lowcount")
    if not os.path.exists(path):
        pytest.skip("no trained low-count weights")
    seed = 6001
    clean, noisy = phantoms.ellipsoids_3d((72, 96, 120), seed=seed, peak=lowcount_peak(seed))
    prof = bg.BM4DProfile(noise_model=bg.NoiseModel.POISSON)
    plain = bg.bmnd(noisy, prof)
    fast = bg.bmnd(noisy, prof, pilot="learned", pilot_weights=path)
    details = {}
    ref = bmnd_fast(cuda.from_numpy(noisy).cuda(), prof, PilotNet.load(path), details=details).cpu().numpy()
    np.testing.assert_allclose(fast, ref, rtol=0, atol=1e-4 * float(np.max(ref)))
    p_noisy, p_plain, p_fast = (phantoms.psnr(v, clean) for v in (noisy, plain, fast))
    print(f"low-count {noisy.shape}: noisy {p_noisy:.3f} dB, plain {p_plain:.3f} dB, fast {p_fast:.3f} dB, "
          f"fallback tiles {details['fallback_tiles']} of {details['tiles']}")
    assert p_fast >= p_plain - 0.4, (p_fast, p_plain)
    assert p_fast > p_noisy + 12.0, (p_fast, p_noisy)
    assert 0 <= details["fallback_tiles"] <= details["tiles"]
