"""bmnd_stage_noalloc: the allocation-free stage entry point.

Some callers may not allocate device memory once they are running (a host
whose memory pool owns the device, a binding without access to the CUDA
allocator).  bmnd_stage_noalloc serves them with a fixed scratch array
compiled into the library instead of a caller workspace.  This test calls it
through the C ABI twice in a row and checks both results against bmnd_stage
with a caller-provided workspace, within the tolerance of the parity tests
(1e-3 counts), and that an oversized stage is refused before any device work.
This file is collected last so a failure here leaves the other results intact.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-3


def _stage_inputs(stage, noisy, profile):
    from bmnd_gb300 import plan
    from bmnd_gb300.validation import resolve_profile

    res = resolve_profile(profile, noisy.shape)
    p = plan.stage_params(profile, noisy.shape, stage, res.blockmatch_distance, res.variance_k)
    block = tuple(getattr(profile, f"{stage}_block_size"))
    counts = tuple(s - b + 1 for s, b in zip(noisy.shape, block))
    sched = plan.reference_schedule(profile, counts, stage)
    return p, np.array(sched.reference_abs, dtype=np.int32)


def _with_workspace(torch, native, p, x, pilot, refs):
    from bmnd_gb300 import _abi

    need = ctypes.c_uint64(0)
    _abi.check(native.bmnd_stage_workspace_bytes(ctypes.byref(p), refs.shape[0], ctypes.byref(need)))
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    out = torch.empty_like(x)
    _abi.check(native.bmnd_stage(ctypes.byref(p), x.data_ptr(), None if pilot is None else pilot.data_ptr(),
                                 refs.data_ptr(), refs.shape[0], out.data_ptr(), None, None, None,
                                 ws.data_ptr(), ws.numel(), 0))
    torch.cuda.synchronize()
    return out


def _no_alloc(torch, native, p, x, pilot, refs):
    from bmnd_gb300 import _abi

    out = torch.empty_like(x)
    allocs = _abi.device_alloc_count()
    _abi.check(native.bmnd_stage_noalloc(ctypes.byref(p), x.data_ptr(),
                                         None if pilot is None else pilot.data_ptr(), refs.data_ptr(),
                                         refs.shape[0], out.data_ptr(), 0))
    torch.cuda.synchronize()
    # the library made no device allocation of its own during the call
    assert _abi.device_alloc_count() == allocs
    return out


@pytest.mark.parametrize("kind", ["bm3d", "bm4d"])
def test_noalloc_stage_matches_workspace_stage(cuda, native, kind):
    import bmnd_gb300 as bg
    from bmnd_gb300 import phantoms

    if kind == "bm3d":
        _, noisy = phantoms.shapes_2d(size=96, seed=21)
        make = lambda: bg.BM3DProfile(noise_model="poisson")  # noqa: E731
    else:
        _, noisy = phantoms.ellipsoids_3d(size=24, seed=22, count=8)
        make = lambda: bg.BM4DProfile(noise_model="poisson")  # noqa: E731
    x = cuda.from_numpy(noisy).cuda()
    pilot = None
    for stage in ("ht", "wiener"):
        p, refs_h = _stage_inputs(stage, noisy, make())
        refs = cuda.from_numpy(refs_h).cuda()
        want = _with_workspace(cuda, native, p, x, pilot, refs).cpu().numpy()
        first = _no_alloc(cuda, native, p, x, pilot, refs).cpu().numpy()
        second = _no_alloc(cuda, native, p, x, pilot, refs).cpu().numpy()
        assert np.max(np.abs(first - want)) <= TOL, (stage, float(np.max(np.abs(first - want))))
        assert np.max(np.abs(second - want)) <= TOL, (stage, float(np.max(np.abs(second - want))))
        pilot = cuda.from_numpy(want).cuda()


@pytest.mark.parametrize("precision", ["approx", "subsampled"])
def test_noalloc_screening_precisions_match_workspace_stage(cuda, native, precision):
    """The Wiener stage with the screening forms of matching (approximate and
    subsampled): their per-voxel arrays come from the fixed array, as they come
    from the workspace in bmnd_stage, so both entry points give the same match
    sets and estimates, twice in a row."""
    import bmnd_gb300 as bg
    from bmnd_gb300 import _abi, phantoms
    from bmnd_gb300.api import stage_device

    _, noisy = phantoms.ellipsoids_3d(size=24, seed=23, count=8)
    x = cuda.from_numpy(noisy).cuda()
    prof = bg.BM4DProfile(noise_model="poisson")
    pilot = stage_device(x, prof, "ht")
    p, refs_h = _stage_inputs("wiener", noisy, prof)
    p.match_precision = _abi.MATCH_APPROX if precision == "approx" else _abi.MATCH_SUBSAMPLED
    refs = cuda.from_numpy(refs_h).cuda()
    want = _with_workspace(cuda, native, p, x, pilot, refs).cpu().numpy()
    for _ in range(2):
        got = _no_alloc(cuda, native, p, x, pilot, refs).cpu().numpy()
        assert np.max(np.abs(got - want)) <= TOL, (precision, float(np.max(np.abs(got - want))))


def test_noalloc_rejects_oversized_stage(cuda, native):
    import bmnd_gb300 as bg
    from bmnd_gb300 import _abi

    shape = (2048, 2048)  # 16 B/voxel of accumulators alone exceed the 64 MiB array
    p, refs_h = _stage_inputs("ht", np.zeros(shape, dtype=np.float32), bg.BM3DProfile(noise_model="poisson"))
    x = cuda.zeros(shape, dtype=cuda.float32, device="cuda")
    refs = cuda.from_numpy(refs_h).cuda()
    out = cuda.empty_like(x)
    rc = native.bmnd_stage_noalloc(ctypes.byref(p), x.data_ptr(), None, refs.data_ptr(), refs_h.shape[0],
                                   out.data_ptr(), 0)
    assert rc == _abi.ERR_WORKSPACE
    assert b"static scratch" in native.bmnd_last_error()
