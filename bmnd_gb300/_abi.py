"""ctypes view of the C ABI in include/bmnd_gb300.h and the library loader.

The library (``bmnd_gb300/libbmnd_gb300.so``) is built in-tree by
:mod:`bmnd_gb300.build`.  There is no fallback: if it is missing or was built
for another ABI version, :func:`lib` raises ``RuntimeError``.
"""

from __future__ import annotations

import ctypes
import os
import threading

ABI_VERSION = 3
MAX_DIMS = 3
MAX_EDGE = 8
MAX_PATCH = 512
MAX_STACK = 32

OK = 0
ERR_INVALID_ARG = -1
ERR_UNSUPPORTED = -2
ERR_WORKSPACE = -3
ERR_CUDA = -4
ERR_TIMEOUT = -5

DIST_SSD = 0
DIST_POISSON_DEVIANCE = 1
DIST_PEARSON = 2
DIST_ANSCOMBE_SSD = 3

FILTER_HARD_THRESHOLD = 0
FILTER_WIENER = 1

GROUP_HAAR = 0
GROUP_DCT = 1
GROUP_NONE = 2

WEIGHT_CLASSIC = 0
WEIGHT_VARIANCE = 1
WEIGHT_RISK = 2

GAIN_VARIANCE_SCALED = 0
GAIN_CLASSIC = 1
GAIN_NOISE_FLOOR = 2
POLICY_FIXED = 0
POLICY_REFERENCE_FINITE_COUNT = 1
POLICY_CANDIDATE_STANDARDIZED = 2
SOURCE_PILOT = 0
SOURCE_OBSERVATION = 1

NOISE_POISSON = 0
NOISE_GAUSSIAN = 1

MATCH_EXACT = 0
MATCH_FAST = 1
MATCH_APPROX = 2
MATCH_SUBSAMPLED = 3
CONV_TCGEN05 = 0
CONV_MMA_SYNC = 1

STATIC_SCRATCH_BYTES = 64 << 20

_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_F32P = ctypes.POINTER(ctypes.c_float)
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_U64P = ctypes.POINTER(ctypes.c_uint64)


class MatchParams(ctypes.Structure):
    _fields_ = [
        ("ndim", _I32),
        ("counts", _I32 * MAX_DIMS),
        ("search_radius", _I32 * MAX_DIMS),
        ("max_matches", _I32),
        ("min_matches", _I32),
        ("prefer_power_of_two", _I32),
        ("distance", _I32),
        ("stabilize_ties", _I32),
        ("precision", _I32),
        ("count_scale", ctypes.c_double),
    ]


class StageParams(ctypes.Structure):
    _fields_ = [
        ("ndim", _I32),
        ("shape", _I32 * MAX_DIMS),
        ("block", _I32 * MAX_DIMS),
        ("search_radius", _I32 * MAX_DIMS),
        ("max_stack", _I32),
        ("min_stack", _I32),
        ("distance", _I32),
        ("stabilize_ties", _I32),
        ("match_precision", _I32),
        ("filter", _I32),
        ("group_transform", _I32),
        ("variance_k", _I32),
        ("weight_model", _I32),
        ("windowed_synthesis", _I32),
        ("match_threshold", ctypes.c_float),
        ("ht_lambda", ctypes.c_float),
        ("wiener_scale", ctypes.c_float),
        ("reserved0", ctypes.c_float),
        ("count_scale", ctypes.c_double),
        ("variance_floor", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("spatial_fwd", (ctypes.c_float * (MAX_EDGE * MAX_EDGE)) * MAX_DIMS),
        ("spatial_inv", (ctypes.c_float * (MAX_EDGE * MAX_EDGE)) * MAX_DIMS),
        ("window", ctypes.c_float * MAX_PATCH),
        ("spatial_metric_diag", ctypes.c_double * MAX_PATCH),
        ("noise_model", _I32),
        ("cov_domain", _I32 * MAX_DIMS),
        ("cov_maps", ctypes.c_void_p),
        ("match_noise_ssd", ctypes.c_void_p),
        ("ssd_gamma", ctypes.c_float),
        ("ssd_poisson_bias", _I32),
        ("ssd_threshold", ctypes.c_double),
        ("mass_conserve", _I32),
        ("wiener_gain_mode", _I32),
        ("wiener_variance_source", _I32),
        ("wiener_match_source", _I32),
        ("soft_threshold", _I32),
        ("match_policy", _I32),
        ("null_max_count", _I32),
        ("null_moments", ctypes.c_void_p),
        ("policy_beta", ctypes.c_double),
        ("policy_power", ctypes.c_double),
        ("weight_group_scope", _I32),
        ("fast_group_transform", _I32),
        ("exact_risk_weights", _I32),
        ("exact_source_variance", ctypes.c_float),
    ]


class PilotNet(ctypes.Structure):
    _fields_ = [
        ("ndim", _I32),
        ("channels", _I32),
        ("layers", _I32),
        ("batch", _I32),
        ("shape", _I32 * MAX_DIMS),
    ]


_PNP = ctypes.POINTER(PilotNet)
_VP = ctypes.c_void_p

# name -> (restype, argtypes); every symbol include/bmnd_gb300.h declares
SIGNATURES = {
    "bmnd_abi_version": (_I32, []),
    "bmnd_last_error": (ctypes.c_char_p, []),
    "bmnd_launch_count": (_I32, [_U64P]),
    "bmnd_device_alloc_count": (_I32, [_U64P]),
    "bmnd_host_memory_direct": (_I32, [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "bmnd_reference_schedule": (
        _I32,
        [_I32, _I32P, _I32P, _I32P, ctypes.c_double, _I32, _I32P, _I32P, _I32P, _I64, _I64P],
    ),
    "bmnd_blockmatch_patches": (
        _I32,
        [ctypes.POINTER(MatchParams), ctypes.c_void_p, _I32, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _U64],
    ),
    "bmnd_blockmatch_volume": (
        _I32,
        [ctypes.POINTER(MatchParams), ctypes.c_void_p, _I32P, _I32P, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _U64],
    ),
    "bmnd_blockmatch_volume_biased": (
        _I32,
        [ctypes.POINTER(MatchParams), ctypes.c_void_p, _I32P, _I32P, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         _U64],
    ),
    "bmnd_blockmatch_volume_poisson_biased": (
        _I32,
        [ctypes.POINTER(MatchParams), ctypes.c_void_p, _I32P, _I32P, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _U64],
    ),
    "bmnd_stage_workspace_bytes": (_I32, [ctypes.POINTER(StageParams), _I64, _U64P]),
    "bmnd_stage": (
        _I32,
        [ctypes.POINTER(StageParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
         _U64, _U64],
    ),
    "bmnd_stage_sigma_workspace_bytes": (_I32, [ctypes.POINTER(StageParams), _I64, _U64P]),
    "bmnd_stage_sigma": (
        _I32,
        [ctypes.POINTER(StageParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _I64,
         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_void_p, _U64, _U64],
    ),
    "bmnd_stage_noalloc": (
        _I32,
        [ctypes.POINTER(StageParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _I64,
         ctypes.c_void_p, _U64],
    ),
    "bmnd_group_probe_workspace_bytes": (_I32, [ctypes.POINTER(StageParams), _U64P]),
    "bmnd_group_probe": (
        _I32,
        [ctypes.POINTER(StageParams), _VP, _VP, _VP, _VP, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _U64, _U64],
    ),
    "bmnd_unit_rates": (_I32, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _VP, _U64]),
    "bmnd_mma_rates": (_I32, [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                              ctypes.POINTER(ctypes.c_double), _VP, _U64]),
    "bmnd_pilotnet_param_count": (_I32, [_PNP, _I64P]),
    "bmnd_pilotnet_packed_bytes": (_I32, [_PNP, _U64P]),
    "bmnd_pilotnet_workspace_bytes": (_I32, [_PNP, _I32, _U64P]),
    "bmnd_pilotnet_pack": (_I32, [_PNP, _VP, _VP, _U64]),
    "bmnd_pilotnet_status": (_I32, [_PNP, _VP, _U64]),
    "bmnd_pilotnet_set_conv_engine": (_I32, [_I32]),
    "bmnd_pilotnet_set_wait_probe": (_I32, [ctypes.c_uint64]),
    "bmnd_pilotnet_get_conv_engine": (_I32, [_I32P]),
    "bmnd_pilotnet_forward": (_I32, [_PNP, _VP, _VP, _VP, _VP, _VP, _U64, _U64]),
    "bmnd_pilotnet_gradient": (_I32, [_PNP, _VP, _VP, _VP, _VP, _VP, _VP, _U64, _U64]),
    "bmnd_pilotnet_adam": (_I32, [_I64, _VP, _VP, _VP, _VP, _I32, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_float, _VP, _U64]),
    "bmnd_pilot_tile_deviance": (_I32, [_I32, _I32, _I32P, _I32, _VP, _VP, _VP, _I32, ctypes.c_float,
                                        ctypes.c_float, _VP, _U64]),
    "bmnd_run": (
        _I32,
        [ctypes.POINTER(StageParams), ctypes.POINTER(StageParams), ctypes.c_void_p,
         ctypes.c_void_p, _I64, ctypes.c_void_p, _I64, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_void_p, _U64, _U64],
    ),
}

LIB_NAME = "libbmnd_gb300.so"
_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), LIB_NAME)


def lib() -> ctypes.CDLL:
    """Load the native library once; raise if it is absent or mismatched."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"{LIB_NAME} is not built ({path} missing); run "
                "`python -c 'import __graft_entry__ as g; g.build()'` or "
                "`python -m bmnd_gb300.build`"
            )
        handle = ctypes.CDLL(path)
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        version = handle.bmnd_abi_version()
        if version != ABI_VERSION:
            raise RuntimeError(f"{LIB_NAME} has ABI version {version}, expected {ABI_VERSION}")
        _lib = handle
        return _lib


class BmndError(RuntimeError):
    """A non-zero status returned by the native library."""

    def __init__(self, code: int, message: str):
        super().__init__(f"bmnd_gb300 native call failed ({code}): {message}")
        self.code = code


def check(code: int) -> None:
    if code != OK:
        msg = lib().bmnd_last_error()
        raise BmndError(code, msg.decode() if msg else "")


def unit_rates(stream=None) -> dict:
    """Measured MUFU lg2 and FP32 FMA issue rates of the current device, per
    second (``bmnd_unit_rates``)."""
    import torch

    sink = torch.zeros(16, dtype=torch.float32, device=torch.cuda.current_device())
    if stream is None:
        stream = torch.cuda.current_stream()
    lg2, ffma = ctypes.c_double(0.0), ctypes.c_double(0.0)
    check(lib().bmnd_unit_rates(ctypes.byref(lg2), ctypes.byref(ffma), sink.data_ptr(), int(stream.cuda_stream)))
    return {"lg2_per_s": lg2.value, "ffma_per_s": ffma.value}


def mma_rates(configs=((16, 2), (48, 1), (48, 2), (96, 2), (128, 2), (256, 2)), stream=None) -> list:
    """Measured clocks per 128 x N x 16 BF16 tcgen05 MMA when `issuers` threads
    of a CTA issue them back to back, for each (N, issuers) in `configs`
    (``bmnd_mma_rates``).  Returns [(N, issuers, clocks), ...]."""
    import torch

    n = len(configs)
    cols = (ctypes.c_int32 * n)(*[int(c[0]) for c in configs])
    iss = (ctypes.c_int32 * n)(*[int(c[1]) for c in configs])
    out = (ctypes.c_double * n)()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    scratch = torch.zeros(sms + 1, dtype=torch.int64, device=torch.cuda.current_device())
    if stream is None:
        stream = torch.cuda.current_stream()
    check(lib().bmnd_mma_rates(n, cols, iss, out, scratch.data_ptr(), int(stream.cuda_stream)))
    return [(int(c[0]), int(c[1]), float(out[i])) for i, c in enumerate(configs)]


def host_memory_direct(device: int) -> bool:
    """True when the device reads ordinary (pageable) host memory through the
    host's page tables, so host copies need no page-locked staging
    (``bmnd_host_memory_direct``)."""
    v = ctypes.c_int32(0)
    check(lib().bmnd_host_memory_direct(int(device), ctypes.byref(v)))
    return bool(v.value)


def device_alloc_count() -> int:
    """Device allocations the native library has made itself since it was loaded."""
    n = ctypes.c_uint64(0)
    check(lib().bmnd_device_alloc_count(ctypes.byref(n)))
    return int(n.value)


def launch_count() -> int:
    """Kernel launches of the native library since it was loaded."""
    n = ctypes.c_uint64(0)
    check(lib().bmnd_launch_count(ctypes.byref(n)))
    return int(n.value)
