"""Benchmark: Mvoxel/s of the BMND direct-Poisson path on one GB300.

Workload (default): 256^3 float32 BM4D-Poisson volume of 30 random ellipsoids
(semi-axes 10-80 voxels, intensities U[5, 30], background 2, Poisson noise;
seeded synthetic data, see bmnd_gb300/phantoms.py) denoised with
BM4DProfile(noise_model="poisson") defaults.  One step = one denoising call.

* ``value``  -- voxels / device time of the learned-pilot fast path
  (pilot.bmnd_fast: the net, the per-tile check, the fast Wiener stage) with
  the input resident in HBM (CUDA events on the launching stream; L2 flushed
  between steps); without trained weights, of the plain path bmnd_device()
  (hard thresholding, then Wiener on its pilot), which is also reported as
  ``plain`` beside the fast path.
* ``e2e``    -- the same path from host memory to host memory: copy in from a
  page-locked buffer, denoise, copy the estimate back.
* ``roofline`` -- the dominant kernel (largest share of the step), timed with
  CUDA events inside this script.
* ``cpu_baseline`` -- the C oracle (the reference algorithm restated in C,
  OpenMP on every host core) on a bounded sample of the same workload.

``--impl reference`` times that CPU implementation alone (rank 0).  Multi-GPU
runs are independent replicas (one volume per rank, weak scaling).
"""

from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mvoxel/s at 256\u00b3 BM4D: learned+BF16 vs plain GPU at \u22640.05 dB PSNR loss"

WORKLOADS = {
    "bm4d256": dict(kind="bm4d", size=256, desc="256^3 BM4D-Poisson, 30 ellipsoids"),
    "bm4d128": dict(kind="bm4d", size=128, desc="128^3 BM4D-Poisson, 30 ellipsoids"),
    "bm3d2048": dict(kind="bm3d", size=2048, desc="2048^2 BM3D-Poisson, 40 blobs + 60 rectangles"),
    "bm3d256": dict(kind="bm3d", size=256, desc="256^2 BM3D-Poisson, 12 rectangles/discs"),
    # stationary Gaussian noise (default profiles, sigma given)
    "gauss2048": dict(kind="bm3d", size=2048, noise="gaussian", sigma=5.0,
                      desc="2048^2 BM3D-Gaussian sigma=5, 40 blobs + 60 rectangles"),
    "gauss256": dict(kind="bm4d", size=256, noise="gaussian", sigma=2.0,
                     desc="256^3 BM4D-Gaussian sigma=2, 30 ellipsoids"),
    "gauss128": dict(kind="bm4d", size=128, noise="gaussian", sigma=2.0,
                     desc="128^3 BM4D-Gaussian sigma=2, 30 ellipsoids"),
}


def is_gaussian(name: str) -> bool:
    return WORKLOADS[name].get("noise") == "gaussian"


def make_input(name: str, seed: int):
    from bmnd_gb300 import phantoms

    w = WORKLOADS[name]
    if w["kind"] == "bm4d":
        clean, noisy = phantoms.ellipsoids_3d(w["size"], seed=seed)
    elif w["size"] == 2048:
        clean, noisy = phantoms.blobs_2d(2048, seed=seed)
    else:
        clean, noisy = phantoms.shapes_2d(w["size"], seed=seed)
    if is_gaussian(name):
        rng = np.random.default_rng(7000 + seed)
        noisy = (clean + w["sigma"] * rng.standard_normal(clean.shape)).astype(np.float32)
    return clean, noisy


def make_profile(name: str):
    import bmnd_gb300 as bg

    cls = bg.BM4DProfile if WORKLOADS[name]["kind"] == "bm4d" else bg.BM3DProfile
    if is_gaussian(name):
        return cls()
    return cls(noise_model=bg.NoiseModel.POISSON)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": float(max(smax)) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def load_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def profile_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


# ---------------------------------------------------------------------------
# CPU baseline (the C oracle on a bounded sample)
# ---------------------------------------------------------------------------
def data_desc(workload: str) -> str:
    if is_gaussian(workload):
        return f"synthetic (seeded phantom, additive Gaussian noise sigma={WORKLOADS[workload]['sigma']})"
    return "synthetic (seeded phantom, Poisson counts)"


def profile_desc(workload: str) -> str:
    name = "BM4DProfile" if WORKLOADS[workload]["kind"] == "bm4d" else "BM3DProfile"
    if is_gaussian(workload):
        return f"{name}() defaults (Gaussian), sigma={WORKLOADS[workload]['sigma']}"
    return f"{name}(noise_model=poisson) defaults"


# The reference package itself, timed once in the build container (x86-64, one
# thread): Numba is not installable there, so it ran as plain Python through the
# import stand-ins of oracle/shim.  The 256^2 BM3D-Poisson image (12 rectangles
# and discs, seed 0) took 2 h 20 min.
REFERENCE_MEASURED = {
    "what": "the reference bmnd() itself, pure Python (Numba unavailable), one thread, x86-64",
    "workload": "256^2 BM3D-Poisson, 12 rectangles/discs, seed 0",
    "seconds": 8400.0,
    "value": 65536 / 8400.0 / 1e6,
    "unit": "Mvoxel/s",
}


def cpu_baseline(workload: str, seed: int, budget_s: float = 20.0) -> dict:
    if is_gaussian(workload):
        return {"value": None, "unit": "Mvoxel/s", "cores": 0, "kind": "none",
                "sample": "the CPU oracle restates the Poisson path only; the Gaussian path is pinned on the "
                          "reference's own outputs (tests/golden/gauss_*.npz)"}
    import oracle

    _, noisy = make_input(workload, seed) if WORKLOADS[workload]["size"] <= 256 else make_input("bm3d256", seed)
    if noisy.ndim == 3:
        crop = 64
        sample = noisy[:crop, :crop, :crop].copy()
        desc = f"{crop}^3 corner crop of the same volume, both stages"
    else:
        crop = 128
        sample = noisy[:crop, :crop].copy()
        desc = f"{crop}^2 corner crop, both stages"
    threads = os.cpu_count() or 1
    oracle.build()
    t0 = time.perf_counter()
    reps = 0
    while True:
        oracle.bmnd(sample, make_profile(workload), threads=threads)
        reps += 1
        if time.perf_counter() - t0 > budget_s or reps >= 3:
            break
    dt = (time.perf_counter() - t0) / reps
    return {
        "value": sample.size / dt / 1e6,
        "unit": "Mvoxel/s",
        "cores": threads,
        "cpu_model": cpu_model(),
        "kind": "port",
        "sample": desc,
        "seconds_per_call": dt,
        "reference_itself": REFERENCE_MEASURED,
    }


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_kernels(torch, noisy_t, profile, reps: int = 2, stages=("ht", "wiener"), pilot=None,
                 precision=None, gauss=None, fast_transforms: bool = False) -> dict:
    """CUDA-event times of the block-matching kernels and of each stage.

    ``pilot`` (optional) is the Wiener stage's pilot; by default it is the
    stage-1 output, as in the plain pipeline.  ``precision`` maps a stage to
    its matching precision (default: exact for stage 1, bounded screening for
    stage 2, which is what the plain pipeline runs)."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import _abi, plan
    from bmnd_gb300.validation import resolve_profile

    L = _abi.lib()
    shape = tuple(noisy_t.shape)
    resolved = resolve_profile(profile, shape)
    stream = torch.cuda.current_stream()
    res = {}
    if precision is None:
        if gauss is not None:
            # SSD: the pipeline's choice (tensor-core screening in 2-D, the exact kernel in 3-D)
            ssd = _abi.MATCH_FAST if len(shape) == 2 else _abi.MATCH_EXACT
            precision = {"ht": ssd, "wiener": ssd}
        else:
            precision = {"ht": _abi.MATCH_EXACT, "wiener": _abi.MATCH_FAST}
    for stage in stages:
        stage_prec = precision[stage]
        p = plan.stage_params(profile, shape, stage, resolved.blockmatch_distance, resolved.variance_k,
                              stage_prec if stage_prec in (_abi.MATCH_APPROX, _abi.MATCH_SUBSAMPLED)
                              else _abi.MATCH_EXACT,
                              None if gauss is None else gauss[stage], fast_transforms=fast_transforms)
        block = tuple(getattr(profile, f"{stage}_block_size"))
        counts = tuple(s - b + 1 for s, b in zip(shape, block))
        sched = plan.reference_schedule(profile, counts, stage)
        n = len(sched)
        refs = torch.from_numpy(np.array(sched.reference_abs, dtype=np.int32)).cuda()
        src = noisy_t if stage == "ht" else pilot
        thr_v = float(p.match_threshold)
        if gauss is not None:
            # SSD threshold: t (max - min)^2 of the matched volume
            span = float(src.max().item() - src.min().item())
            thr_v = float(np.float32(p.ssd_threshold * (span if span > 0 else 1.0) ** 2))
        thr = torch.full((n,), thr_v, device="cuda")
        sel = torch.empty((n, p.max_stack), dtype=torch.int32, device="cuda")
        cnt = torch.empty(n, dtype=torch.int32, device="cuda")
        acc = torch.empty(n, dtype=torch.int32, device="cuda")
        mp = _abi.MatchParams()
        mp.ndim = len(shape)
        for a in range(len(shape)):
            mp.counts[a] = counts[a]
            mp.search_radius[a] = p.search_radius[a]
        mp.max_matches, mp.min_matches, mp.prefer_power_of_two = p.max_stack, p.min_stack, 1
        mp.distance, mp.stabilize_ties, mp.count_scale = p.distance, p.stabilize_ties, p.count_scale
        # the pipeline matches the real-valued pilot with the screened path
        mp.precision = stage_prec
        sh = (ctypes.c_int32 * len(shape))(*shape)
        bl = (ctypes.c_int32 * len(shape))(*block)
        ssd_bias = None if gauss is None else gauss[stage].get("ssd")
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if ssd_bias is not None:
                _abi.check(L.bmnd_blockmatch_volume_biased(
                    ctypes.byref(mp), src.data_ptr(), sh, bl, refs.data_ptr(), n, thr.data_ptr(),
                    ssd_bias.data_ptr(), float(gauss[stage]["gamma"]), sel.data_ptr(), cnt.data_ptr(),
                    acc.data_ptr(), int(stream.cuda_stream)))
            else:
                _abi.check(L.bmnd_blockmatch_volume(ctypes.byref(mp), src.data_ptr(), sh, bl, refs.data_ptr(),
                                                    n, thr.data_ptr(), sel.data_ptr(), cnt.data_ptr(),
                                                    acc.data_ptr(), int(stream.cuda_stream)))
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        nbytes = ctypes.c_uint64(0)
        _abi.check(L.bmnd_stage_workspace_bytes(ctypes.byref(p), n, ctypes.byref(nbytes)))
        ws = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
        out = torch.empty_like(noisy_t)
        stimes = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _abi.check(L.bmnd_stage(ctypes.byref(p), noisy_t.data_ptr(),
                                    None if stage == "ht" else pilot.data_ptr(), refs.data_ptr(), n,
                                    out.data_ptr(), None, None, None, ws.data_ptr(), ws.numel(),
                                    int(stream.cuda_stream)))
            e1.record(stream)
            e1.synchronize()
            stimes.append(e0.elapsed_time(e1))
        counts_h = cnt.cpu().numpy()
        if stage == "ht":
            pilot = out
        # candidate pairs actually scored (clipped windows) -> deviance voxel-terms
        refs_h = np.array(sched.reference_abs, dtype=np.int64)
        pairs = np.ones(n, dtype=np.int64)
        for a in range(len(shape)):
            lo = np.maximum(refs_h[:, a] - p.search_radius[a], 0)
            hi = np.minimum(refs_h[:, a] + p.search_radius[a], counts[a] - 1)
            pairs *= hi - lo + 1
        P = int(np.prod(block))
        terms = int(pairs.sum()) * P
        if stage_prec == _abi.MATCH_SUBSAMPLED:
            # the even sub-lattice for every candidate, the full patch for 4 K of them
            ps = int(np.prod([(b + 1) // 2 for b in block]))
            terms = int(pairs.sum()) * ps + n * min(4 * p.max_stack, 512) * P
        res[stage] = {
            "match_ms": float(np.median(times)),
            "stage_ms": float(np.median(stimes)),
            "groups": n,
            "pairs": int(pairs.sum()),
            "voxel_terms": terms,
            "mean_group": float(counts_h.mean()),
            "P": P,
        }
    return res


def run_config(args, shape, world: int, fast: bool) -> dict:
    """The workload and the settings of the path ``value`` measures."""
    cfg = {
        "workload": WORKLOADS[args.workload]["desc"],
        "shape": list(shape),
        "profile": profile_desc(args.workload),
        "parallelism": f"replicas{world}",
        "l2": "flushed between timed steps (256 MiB write)",
    }
    if fast:
        from bmnd_gb300 import pilot as pl

        nd = len(shape)
        stage2 = dict(pl.FAST_STAGE2[nd])
        cfg.update({
            "path": "bmnd(volume, profile, pilot='learned')",
            "pilot": "learned: residual conv net, BF16 weights and activations, FP32 accumulation, tcgen05 "
                     "implicit GEMM; per-tile Poisson-deviance fallback to the plain stage 1",
            "wiener_step": list(stage2.get("wiener_step", ())) or "profile default",
            "wiener_variance_k": stage2.get("k", "profile default (4)"),
            "wiener_match_precision": pl.FAST_MATCH_PRECISION,
            "wiener_group_transform": "Haar by its sum pyramid",
            "plain_reported_beside": "bmnd(volume, profile) with match_precision "
                                     f"{args.precision!r}: exact FP32 matching, k = 4",
        })
    else:
        cfg.update({"path": "bmnd(volume, profile)", "match_precision": args.precision})
    return cfg


def cpu_model() -> str:
    """The host CPU's model name (lscpu), or the platform string."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return platform.processor() or platform.machine()


def max_over_ranks(values, dist, device: str) -> list[float]:
    """Element-wise maximum of per-rank floats over all ranks.  Every rank calls
    it; ``dist`` None means a single rank.  ``device`` holds the reduction
    tensor: "cuda" under NCCL, "cpu" under gloo."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def run_gpu(args, rank: int, world: int) -> dict | None:
    import torch

    import bmnd_gb300 as bg
    from bmnd_gb300 import _abi

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl")
        dist = dist_mod
    clean, noisy = make_input(args.workload, seed=rank)
    profile = make_profile(args.workload)
    x = torch.from_numpy(noisy).cuda()
    nvox = noisy.size
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def timed_loop(fn, counts=None):
        """W untimed calls, then K calls each bracketed by CUDA events on the
        launching stream, L2 flushed before each; returns (ms per call, last
        output).  ``counts`` (a list) receives the native library's kernel
        launches over the K timed calls.  The garbage collector is paused
        while the K calls run (as ``timeit`` does): a full collection over
        this process's objects takes milliseconds and would stall the host
        between a call's launches."""
        for _ in range(args.warmup):
            res = fn()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        n0 = _abi.launch_count()
        total = 0.0
        gc.collect()
        gc.disable()
        try:
            for _ in range(args.steps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                res = fn()
                e1.record(stream)
                e1.synchronize()
                total += e0.elapsed_time(e1)
        finally:
            gc.enable()
        torch.cuda.synchronize()
        if counts is not None:
            counts.append(_abi.launch_count() - n0)
        t = total / args.steps
        if dist:
            dist.barrier()
            t = max_over_ranks([t], dist, "cuda")[0]
        return t, res

    gauss = None
    sigma = None
    if is_gaussian(args.workload):
        from bmnd_gb300 import api, gaussian
        from bmnd_gb300.validation import resolve_profile

        sigma = WORKLOADS[args.workload]["sigma"]
        model = gaussian.build_model(noisy.shape, profile.nf, sigma=sigma)
        gauss = api.gaussian_tables(model, profile, noisy.shape, resolve_profile(profile, noisy.shape), x.device)

    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    plain_launches = []
    ms, out = timed_loop(lambda: bg.bmnd_device(x, profile, match_precision=args.precision, gauss=gauss),
                         plain_launches)

    # learned-pilot fast path (network trained by bmnd_gb300.train_pilot)
    from bmnd_gb300 import pilot as pl

    kind = WORKLOADS[args.workload]["kind"]
    wpath = pl.default_net_path(kind)
    fast = None
    if os.path.exists(wpath) and gauss is None:
        net = pl.PilotNet.load(wpath)
        fdet = {}
        fast_launches = []
        ms_fast, out_fast = timed_loop(lambda: pl.bmnd_fast(x, profile, net, details=fdet), fast_launches)
        ms_fs2, out_fs2 = timed_loop(lambda: pl.stage_device(
            x, pl.fast_profile(profile), "wiener", pl.stage_device(x, profile, "ht"),
            match_precision=pl.FAST_MATCH_PRECISION))
        fast = dict(ms=ms_fast, out=out_fast, fallback=fdet.get("fallback_tiles"), tiles=fdet.get("tiles"),
                    pilot=fdet.get("pilot"), ms_fs2=ms_fs2, out_fs2=out_fs2, net=net)
    clocks = sampler.stop()

    # end to end through the public API (host array in, host array out), with
    # the garbage collector paused over the timed calls as in timed_loop
    e2e_steps = max(1, args.steps)
    torch.cuda.synchronize()
    gc.collect()
    gc.disable()
    try:
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host_out = bg.bmnd(noisy, profile, match_precision=args.precision, sigma=sigma)
        e2e_s = (time.perf_counter() - t0) / e2e_steps
    finally:
        gc.enable()
    e2e_fast_s = None
    if fast is not None:
        # the public call a user makes: NumPy array in, NumPy array out, with the
        # argument checks, the copy to the device and the copy back inside
        bg.bmnd(noisy, profile, pilot="learned")
        torch.cuda.synchronize()
        gc.collect()
        gc.disable()
        try:
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                host_fast = bg.bmnd(noisy, profile, pilot="learned")
            e2e_fast_s = (time.perf_counter() - t0) / e2e_steps
        finally:
            gc.enable()
        assert host_fast.shape == noisy.shape
    if dist:
        e2e_s, e2e_fast_max = max_over_ranks([e2e_s, e2e_fast_s or 0.0], dist, "cuda")
        e2e_fast_s = e2e_fast_max if fast is not None else None
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None

    from bmnd_gb300.phantoms import psnr

    kt = time_kernels(torch, x, profile, gauss=gauss)
    peaks = load_peaks()
    from bmnd_gb300 import _abi

    # the compute bounds, measured on this GPU now: MUFU lg2 and FP32 FMA issue rates
    rates = _abi.unit_rates()
    fp32_peak = 2.0 * rates["ffma_per_s"]  # FP32 flops per second (an FMA is two)

    # kernels of the measured path: the fast path when it ran (its Wiener
    # stage on the learned pilot, and the net), else the plain path
    cands = []
    if fast is not None:
        fprof = pl.fast_profile(profile)
        kf = time_kernels(torch, x, fprof, stages=("wiener",), pilot=fast["pilot"],
                          precision={"wiener": bg.api._MATCH_PRECISIONS[pl.FAST_MATCH_PRECISION]},
                          fast_transforms=True)
        kt["fast_wiener"] = kf["wiener"]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            fast["net"].forward(x)
        e1.record(stream)
        e1.synchronize()
        kt["pilot_net_ms"] = e0.elapsed_time(e1) / 3
        k = kf["wiener"]
        cands.append((k["match_ms"], f"blockmatch_wiener_{pl.FAST_MATCH_PRECISION}", "fast_wiener"))
        cands.append((k["stage_ms"] - k["match_ms"], "groupfilter_wiener_fast", "fast_wiener"))
        cands.append((kt["pilot_net_ms"], "pilot_net", None))
    else:
        for stage in ("ht", "wiener"):
            k = kt[stage]
            cands.append((k["match_ms"], f"blockmatch_{stage}", stage))
            cands.append((k["stage_ms"] - k["match_ms"], f"groupfilter_{stage}", stage))
    dom_ms, dom_name, dom_stage = max(cands)
    if dom_name == "pilot_net":
        # the C -> C layers: 2 * taps * C * C flops per voxel each
        nd = noisy.ndim
        C, L_ = fast["net"].channels, fast["net"].layers
        flops = 2.0 * nvox * (3 ** nd) * C * C * (L_ - 2)
        achieved = flops / (dom_ms * 1e-3) / 1e12
        bound, unit, peak_v, alg_bytes = "tensor", "TFLOP/s", peaks["bf16_tflops"], None
        compute = {"what": "BF16 multiply-adds of the C->C layers on the tensor cores"}
    else:
        k = kt[dom_stage]
        wiener = "wiener" in dom_stage
        if dom_name.startswith("blockmatch"):
            # algorithmic bytes: read the matching source once, write the match table
            stack = int(profile.wiener_max_stack_size if wiener else profile.ht_max_stack_size)
            alg_bytes = nvox * 4 + k["groups"] * (stack + 2) * 4
            compute = {
                "what": "SSD voxel terms" if gauss is not None else "Poisson-deviance voxel terms",
                "achieved_gterms_s": k["voxel_terms"] / (dom_ms * 1e-3) / 1e9,
            }
            if dom_name in ("blockmatch_wiener_approx", "blockmatch_wiener_subsampled"):
                # one MUFU lg2 per term: the measured lg2 issue rate bounds the terms per second
                sfu = rates["lg2_per_s"]
                compute["sfu_bound_gterms_s"] = sfu / 1e9
                compute["sfu_bound_source"] = "measured (bmnd_unit_rates: lg2.approx.ftz.f32 chains on every SM)"
                compute["frac_of_sfu_bound"] = k["voxel_terms"] / (dom_ms * 1e-3) / sfu
        else:
            # read noisy (+ pilot) once, write float64 numerator and denominator once
            alg_bytes = nvox * (8 if wiener else 4) + nvox * 16
            kk = min(int(fprof.k) if dom_stage == "fast_wiener" else 4, int(k["mean_group"]))
            if kk == 0 and gauss is None:
                # no exact planes: the separable transforms dominate.  Per group four
                # passes (observation, pilot, squared variance forward; inverse), each
                # n P (sum of the patch edges) spatial multiply-adds plus the group axis:
                # n^2 P as a matrix product, about 3 n P by the fast path's sum pyramid
                n_ = k["mean_group"]
                edges = float(sum(getattr(fprof if dom_stage == "fast_wiener" else profile, "wiener_block_size")))
                group_macs = 3 * n_ * k["P"] if dom_stage == "fast_wiener" else n_ * n_ * k["P"]
                macs = k["groups"] * 4 * (n_ * k["P"] * edges + group_macs)
                compute = {
                    "what": "separable transform multiply-adds (four passes per group)",
                    "achieved_tmacs_s": macs / (dom_ms * 1e-3) / 1e12,
                    "fp32_ops_frac_of_peak": 2 * macs / (dom_ms * 1e-3) / fp32_peak,
                }
            elif gauss is not None:
                n_ = k["mean_group"]
                terms = k["groups"] * (n_ * (n_ + 1) / 2) * k["P"] * kk
                compute = {
                    "what": "Gaussian exact planes: member pairs x coefficients x planes (one covariance-map "
                            "load and two FP32 multiply-adds each)",
                    "achieved_gterms_s": terms / (dom_ms * 1e-3) / 1e9,
                }
            else:
                pairs = k["groups"] * k["mean_group"] * k["P"] * kk * k["P"]
                compute = {
                    "what": "exact overlap-aware variance: entry x coefficient pairs (one FP32 fused multiply-add "
                            "each)",
                    "achieved_gpairs_s": pairs / (dom_ms * 1e-3) / 1e9,
                    "fp32_ops_frac_of_peak": 2 * pairs / (dom_ms * 1e-3) / fp32_peak,
                }
        achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
        bound, unit, peak_v = "hbm", "GB/s", peaks["hbm_gbs"]
    traffic = profile_traffic(dom_name, args.workload)
    launches = plain_launches[0]  # native kernels over the K timed calls
    plain_value = nvox * world / (ms * 1e-3) / 1e6
    psnr_plain = psnr(out.cpu().numpy(), clean)
    if fast is not None:
        psnr_fast = psnr(fast["out"].cpu().numpy(), clean)
        fast_block = {
            "path": "learned pilot (BF16 tensor-core residual net) + per-tile deviance fallback + Wiener stage "
                    f"with reference step 4, approximate Poisson sigma, {pl.FAST_MATCH_PRECISION} screening",
            "value": nvox * world / (fast["ms"] * 1e-3) / 1e6,
            "ms_per_step": fast["ms"],
            "psnr_db": psnr_fast,
            "psnr_loss_db": psnr_plain - psnr_fast,
            "within_0p05_db": bool(psnr_plain - psnr_fast <= 0.05),
            "speedup_vs_plain": ms / fast["ms"],
            "pilot_psnr_db": psnr(fast["pilot"].cpu().numpy(), clean),
            "fallback_tiles": fast["fallback"],
            "tiles": fast["tiles"],
            "e2e_value": nvox * world / e2e_fast_s / 1e6,
            "fast_stage2_only": {
                "what": "plain stage 1 + the fast Wiener stage",
                "value": nvox * world / (fast["ms_fs2"] * 1e-3) / 1e6,
                "psnr_db": psnr(fast["out_fs2"].cpu().numpy(), clean),
            },
        }
        value = fast_block["value"]
        launches = fast_launches[0]
    elif gauss is not None:
        fast_block = {"unavailable": "the learned pilot is trained for Poisson counts only"}
        value = plain_value
    else:
        fast_block = {"unavailable": f"no trained pilot weights at {os.path.relpath(wpath, ROOT)}"}
        value = plain_value
    result = {
        "metric": METRIC if args.workload == "bm4d256" else f"Mvoxel/s at {WORKLOADS[args.workload]['desc']}",
        "value": value,
        "unit": "Mvoxel/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": fast["ms"] if fast is not None else ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": data_desc(args.workload),
        "config": run_config(args, noisy.shape, world, fast is not None),
        "e2e": {
            "value": nvox * world / (e2e_fast_s if fast is not None else e2e_s) / 1e6,
            "unit": "Mvoxel/s",
            "h2d_bytes_per_step": nvox * 4,
            "d2h_bytes_per_step": nvox * 4,
        },
        "plain": {
            "what": "plain FP32 path, bmnd_device with the profile's defaults",
            "value": plain_value,
            "ms_per_step": ms,
            "psnr_db": psnr_plain,
            "e2e_value": nvox * world / e2e_s / 1e6,
        },
        "fast": fast_block,
        "roofline": {
            "kernel": dom_name,
            "bound": bound,
            "achieved": achieved,
            "peak": peak_v,
            "unit": unit,
            "frac": achieved / peak_v,
            "traffic": traffic,
            "peak_source": peaks["source"],
            "ms_per_launch": dom_ms,
            "algorithmic_bytes": alg_bytes,
            "compute": compute,
        },
        "kernels": kt,
        "unit_rates": {"lg2_per_s": rates["lg2_per_s"], "ffma_per_s": rates["ffma_per_s"],
                       "what": "measured by bmnd_unit_rates after the timed steps"},
        "clocks": clocks,
        "gpu_launches": launches,
        "psnr_db": psnr_fast if fast is not None else psnr_plain,
    }
    if not args.skip_cpu:
        result["cpu_baseline"] = cpu_baseline(args.workload, seed=0)
    if dist:
        dist.destroy_process_group()
    return result


def run_reference(args, rank: int, world: int) -> dict | None:
    if rank != 0:
        return None
    if is_gaussian(args.workload):
        return {"impl": "reference", "unavailable": "the CPU oracle restates the Poisson path only"}
    per = []
    for _ in range(args.warmup):
        cpu_baseline(args.workload, seed=0, budget_s=5.0)
    for _ in range(args.steps):
        per.append(cpu_baseline(args.workload, seed=0, budget_s=5.0))
    v = float(np.median([p["value"] for p in per]))
    cb = dict(per[0])
    cb["value"] = v
    return {
        "impl": "reference",
        "metric": METRIC if args.workload == "bm4d256" else f"Mvoxel/s at {WORKLOADS[args.workload]['desc']}",
        "value": v,
        "unit": "Mvoxel/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * float(np.median([p["seconds_per_call"] for p in per])),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded phantom, Poisson counts)",
        "config": {"workload": WORKLOADS[args.workload]["desc"], "sample": cb["sample"]},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "Mvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bm4d256", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="exact", choices=["exact", "fast", "approx"])
    ap.add_argument("--skip-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus))
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_gpu(args, rank, world)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
