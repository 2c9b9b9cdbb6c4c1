"""Train the learned stage-1 pilot on the GPU and evaluate the fast path.

    python -m bmnd_gb300.train_pilot --kind bm4d --out bmnd_gb300/weights/pilot_bm4d.npz

Training pairs are (noisy phantom, plain stage-1 estimate) produced by this
package's own GPU path on seeded synthetic phantoms (seeds 1000 + i); the
held-out evaluation volume uses seed 2000, the benchmark seeds 0 .. 7.  The
net's forward and backward passes are the kernels of ``csrc/pilotnet.cu``.
"""

from __future__ import annotations

import argparse
import json
import os
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--kind", default="bm4d", choices=["bm4d", "bm3d", "bm4d_lowcount", "bm3d_windows"])
    ap.add_argument("--seed0", type=int, default=1000, help="first training phantom seed")
    ap.add_argument("--eval-uneven", action="store_true",
                    help="only evaluate the saved net on eight uneven volumes (128^3 .. 320^3)")
    ap.add_argument("--eval-images", type=int, default=0, metavar="N",
                    help="only evaluate the saved 2-D net on the 2048^2 benchmark images of seeds 0 .. N-1")
    ap.add_argument("--size", type=int, default=None)
    ap.add_argument("--count", type=int, default=8)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--crop", type=int, default=32)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--channels", type=int, default=None)
    ap.add_argument("--layers", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)

    import numpy as np
    import torch

    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.api import stage_device
    from bmnd_gb300.pilot import (PilotNet, bmnd_fast, calibrate_excess_high, default_net_path, fast_profile,
                                  lowcount_peak, training_pairs)

    torch.cuda.set_device(0)
    nd = 2 if args.kind.startswith("bm3d") else 3
    if args.eval_uneven:
        evaluate_uneven(args.kind, args.out or default_net_path(args.kind))
        return
    if args.eval_images:
        evaluate_images(args.out or default_net_path(args.kind), args.eval_images)
        return
    channels = args.channels or (48 if nd == 3 else 32)
    layers = args.layers or (8 if nd == 3 else 10)
    crop = args.crop if nd == 3 else max(args.crop, 64)
    if args.size is None:
        args.size = 256 if nd == 3 else 2048
    t0 = time.time()
    pairs = training_pairs(args.kind, args.size, args.count, seed0=args.seed0)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    net = PilotNet(nd, channels, layers, seed=args.seed)
    t0 = time.time()
    hist = net.fit(pairs, steps=args.steps, crop=crop, batch=args.batch, lr=args.lr, seed=args.seed,
                   log_every=max(args.steps // 20, 1), log=lambda m: print(m, flush=True))
    torch.cuda.synchronize()
    t_train = time.time() - t0
    net.excess_high = calibrate_excess_high(pairs)
    from bmnd_gb300.pilot import tile_excess

    from bmnd_gb300.pilot import default_tile

    ev = np.concatenate([np.ravel(tile_excess(x, t, default_tile(nd))[0]) for x, t in pairs])
    print(f"plain stage-1 tile excess: min {ev.min():.4f} median {np.median(ev):.4f} max {ev.max():.4f}", flush=True)
    out = args.out or default_net_path(args.kind)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    net.save(out)

    # held-out evaluation: pilot quality and the fast path against the plain path
    prof = (bg.BM4DProfile if nd == 3 else bg.BM3DProfile)(noise_model=bg.NoiseModel.POISSON)
    if args.kind == "bm4d_lowcount":
        clean, noisy = phantoms.ellipsoids_3d(args.size, seed=2000, peak=lowcount_peak(2000))
    elif args.kind == "bm3d_windows":
        clean, noisy = phantoms.blobs_2d(2048, seed=2000)  # trained on windows, evaluated on a full image
    elif nd == 3:
        clean, noisy = phantoms.ellipsoids_3d(args.size, seed=2000)
    elif args.size >= 1024:
        clean, noisy = phantoms.blobs_2d(args.size, seed=2000)
    else:
        clean, noisy = phantoms.shapes_2d(args.size, seed=2000)
    x = torch.from_numpy(noisy).cuda()
    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            r = fn()
        e1.record()
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1) / reps

    plain_pilot = stage_device(x, prof, "ht")
    plain, ms_plain = timed(lambda: bg.bmnd_device(x, prof))
    d = {}
    fast, ms_fast = timed(lambda: bmnd_fast(x, prof, net, details=d))
    nocheck, ms_nocheck = timed(lambda: bmnd_fast(x, prof, net, check=False))
    plainpilot_fast = stage_device(x, fast_profile(prof), "wiener", plain_pilot, match_precision="approx")
    learned_pilot, ms_net = timed(lambda: net.forward(x))
    r = dict(
        data_seconds=t_data, train_seconds=t_train, steps=args.steps, crop=crop, batch=args.batch,
        loss_first=hist[0][1], loss_last=hist[-1][1],
        psnr_noisy=phantoms.psnr(noisy, clean),
        psnr_plain_stage1=phantoms.psnr(plain_pilot.cpu().numpy(), clean),
        psnr_learned_pilot=phantoms.psnr(learned_pilot.cpu().numpy(), clean),
        psnr_learned_pilot_vs_plain_stage1=phantoms.psnr(learned_pilot.cpu().numpy(), plain_pilot.cpu().numpy()),
        psnr_plain=phantoms.psnr(plain.cpu().numpy(), clean),
        psnr_fast=phantoms.psnr(fast.cpu().numpy(), clean),
        psnr_fast_no_fallback=phantoms.psnr(nocheck.cpu().numpy(), clean),
        psnr_plain_pilot_fast_stage2=phantoms.psnr(plainpilot_fast.cpu().numpy(), clean),
        ms_plain=ms_plain, ms_fast=ms_fast, ms_fast_no_fallback=ms_nocheck, ms_net=ms_net,
        excess_high=net.excess_high, fallback_tiles=d["fallback_tiles"], tiles=d["tiles"], weights=out,
    )
    print(json.dumps(r), flush=True)


UNEVEN_SEED = 5000


def uneven_shapes(count: int = 8, lo: int = 128, hi: int = 320, seed: int = UNEVEN_SEED):
    """``count`` volume shapes with every extent drawn uniformly from [lo, hi]."""
    import numpy as np

    rng = np.random.default_rng(seed)
    return [tuple(int(v) for v in rng.integers(lo, hi + 1, size=3)) for _ in range(count)]


def evaluate_uneven(kind: str, weights: str) -> list:
    """The fast path with the net in ``weights`` against the plain path on eight
    uneven volumes (30 ellipsoids, seeds 5000 + i; for "bm4d_lowcount" a peak of
    U[2, 5] counts): PSNR against the clean phantom and against the plain
    output, the tiles that fell back, and Mvoxel/s of both paths.  One JSON line
    per volume."""
    import torch

    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.pilot import PilotNet, bmnd_fast, lowcount_peak

    net = PilotNet.load(weights)
    prof = bg.BM4DProfile(noise_model=bg.NoiseModel.POISSON)
    rows = []

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r = fn()
        e1.record()
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1)

    for i, shape in enumerate(uneven_shapes()):
        seed = UNEVEN_SEED + i
        peak = lowcount_peak(seed) if kind == "bm4d_lowcount" else None
        clean, noisy = phantoms.ellipsoids_3d(shape, seed=seed, peak=peak)
        x = torch.from_numpy(noisy).cuda()
        plain, ms_plain = timed(lambda: bg.bmnd_device(x, prof))
        d = {}
        fast, ms_fast = timed(lambda: bmnd_fast(x, prof, net, details=d))
        p_plain = phantoms.psnr(plain.cpu().numpy(), clean)
        p_fast = phantoms.psnr(fast.cpu().numpy(), clean)
        row = dict(shape=list(shape), peak=peak, psnr_noisy=phantoms.psnr(noisy, clean), psnr_plain=p_plain,
                   psnr_fast=p_fast, fast_minus_plain_db=p_fast - p_plain,
                   psnr_fast_vs_plain=phantoms.psnr(fast.cpu().numpy(), plain.cpu().numpy(), float(clean.max())),
                   fallback_tiles=d["fallback_tiles"], tiles=d["tiles"],
                   mvox_s_plain=noisy.size / (ms_plain * 1e-3) / 1e6, mvox_s_fast=noisy.size / (ms_fast * 1e-3) / 1e6,
                   speedup=ms_plain / ms_fast)
        rows.append(row)
        print(json.dumps(row), flush=True)
        del x, plain, fast
        torch.cuda.empty_cache()
    return rows


def evaluate_images(weights: str, count: int, size: int = 2048) -> list:
    """The 2-D fast path with the net in ``weights`` against the plain path on
    the benchmark's blob images (seeds 0 .. count-1): PSNR of both against the
    clean image, the tiles that fell back, and the time of each (CUDA events,
    one warm-up call, the best of three).  One JSON line per image."""
    import torch

    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms
    from bmnd_gb300.pilot import PilotNet, bmnd_fast

    net = PilotNet.load(weights)
    prof = bg.BM3DProfile(noise_model=bg.NoiseModel.POISSON)
    rows = []

    def timed(fn):
        r = fn()
        best = float("inf")
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return r, best

    for seed in range(count):
        clean, noisy = phantoms.blobs_2d(size, seed=seed)
        x = torch.from_numpy(noisy).cuda()
        plain, ms_plain = timed(lambda: bg.bmnd_device(x, prof))
        d = {}
        fast, ms_fast = timed(lambda: bmnd_fast(x, prof, net, details=d))
        p_plain = phantoms.psnr(plain.cpu().numpy(), clean)
        p_fast = phantoms.psnr(fast.cpu().numpy(), clean)
        row = dict(seed=seed, psnr_noisy=phantoms.psnr(noisy, clean), psnr_plain=p_plain, psnr_fast=p_fast,
                   fast_minus_plain_db=p_fast - p_plain, fallback_tiles=d["fallback_tiles"], tiles=d["tiles"],
                   ms_plain=ms_plain, ms_fast=ms_fast, speedup=ms_plain / ms_fast)
        rows.append(row)
        print(json.dumps(row), flush=True)
    return rows


if __name__ == "__main__":
    main()
