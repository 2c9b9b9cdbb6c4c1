"""Host-side logic on CPU: the C ABI library loads, exports every declared
symbol and computes the schedule; transform matrices; profile validation
messages (ported from the reference's pipeline tests)."""

import ctypes
import os
import re

import numpy as np
import pytest

import bmnd_gb300 as bg
from bmnd_gb300 import _abi, plan, transforms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
UNIT = os.path.join(ROOT, "tests", "golden", "unit_reference.npz")


def declared_symbols():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if fname.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fname)).read()
            names |= set(re.findall(r"^\s*(?:int32_t|const char\*|void)\s+(bmnd_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol(native):
    names = declared_symbols()
    assert "bmnd_stage" in names and "bmnd_blockmatch_volume" in names
    for name in names:
        assert hasattr(native, name), name
    assert set(_abi.SIGNATURES) >= names
    assert native.bmnd_abi_version() == _abi.ABI_VERSION


def test_launch_counter_reads_without_a_gpu(native):
    """bmnd_launch_count and bmnd_device_alloc_count need no device."""
    n = _abi.launch_count()
    assert isinstance(n, int) and n >= 0
    assert _abi.launch_count() == n
    a = _abi.device_alloc_count()
    assert isinstance(a, int) and a >= 0
    assert _abi.device_alloc_count() == a


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirrors of the ABI structs have the C compiler's layout."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = []
    for cname, pyname in (("BmndMatchParams", "MatchParams"), ("BmndStageParams", "StageParams")):
        cls = getattr(_abi, pyname)
        lines.append(f'printf("{pyname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{pyname} {field} %zu\\n", offsetof({cname}, {field}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "bmnd_gb300.h"\nint main(void){\n'
                   + "\n".join(lines) + "\nreturn 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for line in out:
        if not line:
            continue
        pyname, field, value = line.split()
        cls = getattr(_abi, pyname)
        got = ctypes.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert got == int(value), (pyname, field, got, value)


@pytest.mark.parametrize("idx", range(6))
def test_native_schedule_matches_reference(native, idx):
    u = np.load(UNIT)
    s = plan._generated_schedule(tuple(int(x) for x in u[f"sched{idx}_counts"]),
                                 tuple(int(x) for x in u[f"sched{idx}_block"]),
                                 tuple(int(x) for x in u[f"sched{idx}_step"]), 2.0, 2)
    np.testing.assert_array_equal(s.reference_abs, u[f"sched{idx}_abs"])
    np.testing.assert_array_equal(s.reference_shifted, u[f"sched{idx}_shifted"])
    np.testing.assert_array_equal(s.shift, u[f"sched{idx}_shift"])


def test_native_errors_are_reported(native):
    n = ctypes.c_int64(0)
    c = (ctypes.c_int32 * 2)(4, 4)
    rc = native.bmnd_reference_schedule(5, c, c, c, 2.0, 2, None, None, None, 0, ctypes.byref(n))
    assert rc == _abi.ERR_INVALID_ARG
    assert b"ndim" in native.bmnd_last_error()
    p = _abi.StageParams()
    out = ctypes.c_uint64(0)
    assert native.bmnd_stage_workspace_bytes(ctypes.byref(p), 10, ctypes.byref(out)) == _abi.ERR_INVALID_ARG


def test_measurement_entries_check_arguments_before_the_device(native):
    """bmnd_mma_rates and bmnd_host_memory_direct reject bad arguments before
    any CUDA call, so the checks run without a GPU."""
    cols = (ctypes.c_int32 * 1)(40)      # not a multiple of 16
    iss = (ctypes.c_int32 * 1)(2)
    out = (ctypes.c_double * 1)()
    sink = ctypes.c_int64(0)
    assert native.bmnd_mma_rates(1, cols, iss, out, ctypes.byref(sink), 0) == _abi.ERR_INVALID_ARG
    assert b"mma rate" in native.bmnd_last_error()
    cols[0], iss[0] = 256, 3            # N x issuers above the 512 tensor-memory columns
    assert native.bmnd_mma_rates(1, cols, iss, out, ctypes.byref(sink), 0) == _abi.ERR_INVALID_ARG
    cols[0], iss[0] = 48, 5             # more issuing threads than warps 0..3
    assert native.bmnd_mma_rates(1, cols, iss, out, ctypes.byref(sink), 0) == _abi.ERR_INVALID_ARG
    assert native.bmnd_mma_rates(1, None, iss, out, ctypes.byref(sink), 0) == _abi.ERR_INVALID_ARG
    assert native.bmnd_mma_rates(0, None, None, None, None, 0) == _abi.OK  # nothing to measure
    assert native.bmnd_host_memory_direct(0, None) == _abi.ERR_INVALID_ARG


def test_transform_matrices_match_reference():
    u = np.load(UNIT)
    for n in (4, 8):
        f, i = transforms.bior15_matrices(n)
        np.testing.assert_array_equal(f, u[f"bior15_fwd_{n}"])
        np.testing.assert_allclose(i, u[f"bior15_inv_{n}"], rtol=0, atol=2e-7)
    for n in (4, 5, 8):
        f, i = transforms.axis_matrices(transforms.TransformType.DCT, n)
        np.testing.assert_array_equal(f, u[f"dct_fwd_{n}"])
        np.testing.assert_array_equal(i, u[f"dct_inv_{n}"])
    for n in (1, 2, 4, 8, 16, 32):
        np.testing.assert_array_equal(transforms.haar_group_matrix(n), u[f"haar_fwd_{n}"])
    for shape in ((8, 8), (4, 4, 4), (5, 5, 5)):
        np.testing.assert_array_equal(plan.kaiser_window(shape, 2.0), u["kaiser_" + "x".join(map(str, shape))])


def _poisson(**kw):
    return bg.BM3DProfile(noise_model="poisson", **kw)


@pytest.mark.parametrize("kwargs,message", [
    (dict(ht_block_size=(8,)), "ht_block_size must contain 2 values"),
    (dict(ht_block_size=(8, 99)), "ht_block_size values cannot exceed volume shape"),
    (dict(ht_step=(0, 3)), "ht_step values must be positive"),
    (dict(wiener_search_window=(-1, 3)), "wiener_search_window values must be non-negative"),
    (dict(ht_min_stack_size=0), "ht_min_stack_size must be a positive integer"),
    (dict(wiener_min_stack_size=40), "wiener_min_stack_size cannot exceed wiener_max_stack_size"),
    (dict(ht_match_threshold=float("nan")), "ht_match_threshold must be finite and non-negative"),
    (dict(k=-1), "k must be a non-negative integer"),
    (dict(poisson_count_scale=0.0), "poisson_count_scale must be finite and positive"),
    (dict(ht_weight_model="risk"), "Unknown ht_weight_model"),
    (dict(blockmatch_distance="nope"), "Unknown blockmatch_distance"),
    (dict(sharpen_alpha=2.0), "Aggregation weighting requires sharpening exponents of 1"),
    (dict(reference_schedule_density=0), "reference_schedule_density must be a positive integer"),
    (dict(ref_batch_size=0), "ref_batch_size must be a positive integer"),
])
def test_profile_validation_messages(kwargs, message):
    vol = np.ones((32, 32), dtype=np.float32)
    with pytest.raises(ValueError, match=re.escape(message)):
        bg.bmnd(vol, _poisson(**kwargs))


def test_input_validation_before_work():
    prof = _poisson()
    with pytest.raises(ValueError, match="sigma and sigma_psd are mutually exclusive"):
        bg.bmnd(np.ones((16, 16)), prof, sigma=1.0, sigma_psd=1.0)
    with pytest.raises(ValueError, match="volume must contain only finite values"):
        bg.bmnd(np.full((16, 16), np.nan), _poisson())
    with pytest.raises(ValueError, match="representable as finite float32"):
        bg.bmnd(np.full((16, 16), 1e300), _poisson())
    with pytest.raises(ValueError, match="only non-negative values"):
        bg.bmnd(-np.ones((16, 16)), _poisson())
    with pytest.raises(ValueError, match="sigma_psd is only supported"):
        bg.bmnd(np.ones((16, 16)), _poisson(), sigma_psd=1.0)
    with pytest.raises(ValueError, match="max_cache_bytes must be a non-negative integer"):
        bg.bmnd(np.ones((16, 16)), _poisson(), max_cache_bytes=-5)
    with pytest.raises(ValueError, match="Unknown noise_model"):
        bg.bmnd(np.ones((16, 16)), bg.BM3DProfile(noise_model="laplace"))


def test_zero_volume_fast_path_needs_no_gpu():
    calls = []
    vol = np.zeros((16, 16), dtype=np.float32)
    out = bg.bmnd(vol, _poisson(), stage_callback=lambda s, e: calls.append((s, e.copy())))
    assert np.array_equal(out, vol) and [c[0] for c in calls] == ["ht", "wiener"]
    out, maps = bg.bmnd(vol, _poisson(), return_sigma_map=True)
    assert set(maps) == {"ht", "wiener"}


def test_profile_enum_coercion_in_place():
    prof = bg.BM4DProfile(noise_model="poisson", blockmatch_distance="poisson_deviance")
    from bmnd_gb300.validation import resolve_profile

    res = resolve_profile(prof, (16, 16, 16))
    assert prof.noise_model is bg.NoiseModel.POISSON
    assert prof.blockmatch_distance is bg.BlockMatchDistance.POISSON_DEVIANCE
    assert res.is_poisson and res.variance_k == 4


def test_unsupported_options_raise_not_implemented():
    vol = np.ones((24, 24), dtype=np.float32)
    with pytest.raises(NotImplementedError):
        bg.bmnd(vol, bg.BM3DProfile(reference_schedule_mode="official"), sigma=1.0)
    # the covariance-aware exact group weighting is limited to patches of <= 128 voxels
    vol3 = np.ones((16, 16, 16), dtype=np.float32)
    with pytest.raises(NotImplementedError):
        bg.bmnd(vol3, bg.BM4DProfile(noise_model="poisson", ht_block_size=(6, 6, 6), ht_weight_scope="group",
                                     ht_weight_domain="windowed_synthesis"))


def test_exact_risk_weight_planning():
    """The covariance-aware exact group weighting is planned exactly when the
    reference takes it (bmndalgo.py:363-370, :752-758): variance or risk
    weights, windowed synthesis, group scope and k > 0; under Gaussian noise
    only when the noise is white (variance.py:1459-1470)."""
    from bmnd_gb300 import gaussian
    from bmnd_gb300.validation import resolve_profile

    shape = (32, 32)
    opts = dict(ht_weight_scope="group", ht_weight_domain="windowed_synthesis", wiener_weight_model="risk",
                wiener_weight_scope="group", wiener_weight_domain="windowed_synthesis")
    for extra, want in ((opts, (1, 1)), (dict(opts, k=0), (0, 0)),
                        (dict(opts, wiener_weight_scope="patch"), (1, 0)),
                        (dict(opts, ht_weight_domain="coefficient"), (0, 1)), ({}, (0, 0))):
        prof = bg.BM3DProfile(noise_model="poisson", **extra)
        res = resolve_profile(prof, shape)
        got = tuple(plan.stage_params(prof, shape, st, res.blockmatch_distance, res.variance_k).exact_risk_weights
                    for st in ("ht", "wiener"))
        assert got == want, (extra, got)
    white = gaussian.build_model(shape, None, sigma=3.0)
    assert abs(gaussian.white_variance(white) - 9.0) < 1e-4
    psd = np.ones(shape, dtype=np.float32)
    psd[0, 1] = 40.0
    colored = gaussian.build_model(shape, None, sigma_psd=psd)
    assert gaussian.white_variance(colored) is None


def test_stage_params_defaults():
    from bmnd_gb300.validation import resolve_profile

    prof = bg.BM4DProfile(noise_model="poisson")
    res = resolve_profile(prof, (32, 32, 32))
    ht = plan.stage_params(prof, (32, 32, 32), "ht", res.blockmatch_distance, res.variance_k)
    wi = plan.stage_params(prof, (32, 32, 32), "wiener", res.blockmatch_distance, res.variance_k)
    assert ht.distance == _abi.DIST_POISSON_DEVIANCE and ht.group_transform == _abi.GROUP_HAAR
    assert list(ht.block) == [4, 4, 4] and list(wi.block) == [5, 5, 5]
    assert ht.max_stack == 16 and wi.max_stack == 32 and ht.variance_k == 4
    assert abs(ht.match_threshold - 2.9527) < 1e-6 and abs(wi.match_threshold - 0.7689) < 1e-6
    assert abs(ht.ht_lambda - 3.0) < 1e-7 and abs(wi.wiener_scale - 0.4) < 1e-7


def test_poisson_ssd_bias_parameters():
    """The planner asks for the Poisson SSD noise bias in hard thresholding only,
    with SSD matching and gamma != 0, gamma as float32 (bmndalgo.py:292-294,
    blockmatching.py:244-262); the library's stage validation rejects an
    inconsistent request before any launch (no GPU needed)."""
    import ctypes

    from bmnd_gb300.enums import BlockMatchDistance
    from bmnd_gb300.validation import resolve_profile

    shape = (32, 32)
    prof = bg.BM3DProfile(noise_model="poisson", blockmatch_distance="ssd", gamma=2.5)
    res = resolve_profile(prof, shape)
    assert res.blockmatch_distance is BlockMatchDistance.SSD
    ht = plan.stage_params(prof, shape, "ht", res.blockmatch_distance, res.variance_k)
    wi = plan.stage_params(prof, shape, "wiener", res.blockmatch_distance, res.variance_k)
    assert ht.distance == _abi.DIST_SSD and ht.ssd_poisson_bias == 1 and ht.ssd_gamma == np.float32(2.5)
    assert wi.ssd_poisson_bias == 0
    for other in (bg.BM3DProfile(noise_model="poisson", blockmatch_distance="ssd", gamma=0.0),
                  bg.BM3DProfile(noise_model="poisson")):
        r = resolve_profile(other, shape)
        assert plan.stage_params(other, shape, "ht", r.blockmatch_distance, r.variance_k).ssd_poisson_bias == 0

    L = _abi.lib()
    nbytes = ctypes.c_uint64(0)
    assert L.bmnd_stage_workspace_bytes(ctypes.byref(ht), 8, ctypes.byref(nbytes)) == _abi.OK
    bad = plan.stage_params(prof, shape, "ht", res.blockmatch_distance, res.variance_k)
    bad.distance = _abi.DIST_POISSON_DEVIANCE
    assert L.bmnd_stage_workspace_bytes(ctypes.byref(bad), 8, ctypes.byref(nbytes)) != _abi.OK
    bad = plan.stage_params(prof, shape, "ht", res.blockmatch_distance, res.variance_k)
    bad.ssd_gamma = float("nan")
    assert L.bmnd_stage_workspace_bytes(ctypes.byref(bad), 8, ctypes.byref(nbytes)) != _abi.OK
    bad = plan.stage_params(prof, shape, "ht", res.blockmatch_distance, res.variance_k)
    bad.ssd_poisson_bias = 2
    assert L.bmnd_stage_workspace_bytes(ctypes.byref(bad), 8, ctypes.byref(nbytes)) != _abi.OK
