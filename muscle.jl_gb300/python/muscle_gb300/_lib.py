"""ctypes binding of libmuscle_gb300.so (declarations in include/muscle_gb300.h).

Loading never falls back to anything: if the shared library is missing or a
symbol is absent, the import of the compute entry points raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from ._build import LIB_PATH

MAX_RANK = 16

OK = 0
ERR_ARGUMENT = 1
ERR_DIMENSION_MISMATCH = 2
ERR_UNSUPPORTED = 3
ERR_WORKSPACE = 4
ERR_CUDA = 5
ERR_DEVICE_TIMEOUT = 6
ERR_OUT_OF_MEMORY = 7
ERR_NOT_FINITE = 8

# Size of the library's fixed scratch array behind mgb_contract_noalloc
# (MGB_NOALLOC_SCRATCH_BYTES in the header; a host test keeps the two equal).
NOALLOC_SCRATCH_BYTES = 32 << 20

F32, F64, C32, C64 = 0, 1, 2, 3
SVD_NORMALIZE, SVD_CONJ_V, SVD_SQRT_S = 1, 2, 4
FORM_AUTO, FORM_PLAIN, FORM_OZAKI, FORM_BF16X3 = 0, 1, 2, 3

FORMS = {"auto": FORM_AUTO, "plain": FORM_PLAIN, "ozaki": FORM_OZAKI, "bf16x3": FORM_BF16X3}

# Every C entry point the header declares, with its ctypes signature.
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_u64 = ctypes.c_uint64


class TensorDesc(ctypes.Structure):
    _fields_ = [
        ("dtype", ctypes.c_int32),
        ("rank", ctypes.c_int32),
        ("modes", ctypes.POINTER(ctypes.c_int32)),
        ("extents", ctypes.POINTER(ctypes.c_int64)),
        ("strides", ctypes.POINTER(ctypes.c_int64)),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int64),
        ("n", ctypes.c_int64),
        ("k", ctypes.c_int64),
        ("batch", ctypes.c_int64),
        ("form", ctypes.c_int32),
        ("slices", ctypes.c_int32),
        ("compute_dtype", ctypes.c_int32),
        ("permute_a", ctypes.c_int32),
        ("permute_b", ctypes.c_int32),
        ("permute_c", ctypes.c_int32),
        ("flops", ctypes.c_double),
        ("workspace_bytes", ctypes.c_uint64),
    ]


class AdaptiveReport(ctypes.Structure):
    _fields_ = [
        ("slices", ctypes.c_int32),
        ("nonfinite", ctypes.c_int32),
        ("estimate", ctypes.c_double * 9),
        ("tolerance", ctypes.c_double),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("rejected", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("pending", ctypes.c_uint64),
        ("used_bytes", ctypes.c_uint64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("elapsed_s", ctypes.c_double),
    ]


_P = ctypes.POINTER
SIGNATURES = {
    "mgb_contraction_plan": (_i32, [_P(_vp), _P(TensorDesc), _P(TensorDesc), _P(TensorDesc), _i32, _i32]),
    "mgb_contract": (_i32, [_vp, _vp, _vp, _vp, _vp, _u64, _vp]),
    "mgb_contract_noalloc": (_i32, [_vp, _vp, _vp, _vp, _vp]),
    "mgb_unary_plan": (_i32, [_P(_vp), _P(TensorDesc), _P(TensorDesc)]),
    "mgb_unary": (_i32, [_vp, _vp, _vp, _vp, _u64, _vp]),
    "mgb_permute": (_i32, [_P(TensorDesc), _P(TensorDesc), _vp, _vp, _vp]),
    "mgb_hadamard": (_i32, [_P(TensorDesc), _P(TensorDesc), _P(TensorDesc), _vp, _vp, _vp, _vp]),
    "mgb_plan_info_get": (_i32, [_vp, _P(PlanInfo)]),
    "mgb_plan_workspace_size": (_i32, [_vp, _P(_u64)]),
    "mgb_plan_destroy": (_i32, [_vp]),
    "mgb_plan_set_timing": (_i32, [_vp, _i32]),
    "mgb_plan_set_band": (_i32, [_vp, _i32]),
    "mgb_plan_operands_swapped": (_i32, [_vp, _P(_i32)]),
    "mgb_plan_timing": (_i32, [_vp, _P(ctypes.c_float), _P(ctypes.c_float)]),
    "mgb_plan_set_tolerance": (_i32, [_vp, ctypes.c_double]),
    "mgb_plan_adaptive_report": (_i32, [_vp, _vp, _vp, _P(AdaptiveReport)]),
    "mgb_group_create": (_i32, [_P(_vp), _P(_vp), _i32, _P(_vp), _P(_vp), _P(_vp)]),
    "mgb_group_update": (_i32, [_vp, _P(_vp), _P(_vp), _P(_vp)]),
    "mgb_group_workspace_size": (_i32, [_vp, _P(_u64)]),
    "mgb_group_execute": (_i32, [_vp, _vp, _u64, _vp]),
    "mgb_group_set_tiles": (_i32, [_vp, _P(_i32)]),
    "mgb_group_execute_part": (_i32, [_vp, _i32, _i32, _vp, _u64, _vp]),
    "mgb_group_prepare_part": (_i32, [_vp, _i32, _i32, _vp, _u64, _vp]),
    "mgb_group_finish": (_i32, [_vp, _vp, _u64, _vp]),
    "mgb_group_destroy": (_i32, [_vp]),
    "mgb_server_create": (_i32, [_P(_vp), _u64, _i32, _i32]),
    "mgb_server_submit": (_i32, [_vp, _vp, _vp, _vp, _vp, _u64, _vp, _P(ctypes.c_int64)]),
    "mgb_server_wait": (_i32, [_vp, ctypes.c_int64, ctypes.c_double, _P(_i32)]),
    "mgb_server_get_stats": (_i32, [_vp, _P(ServerStats)]),
    "mgb_server_reset_stats": (_i32, [_vp]),
    "mgb_server_destroy": (_i32, [_vp]),
    "mgb_last_error": (ctypes.c_char_p, []),
    "mgb_device_status": (_i32, [_vp, _P(_i32)]),
    "mgb_selftest_wait_timeout": (_i32, [_vp]),
    "mgb_version": (ctypes.c_char_p, []),
    "mgb_probe_fp64": (_i32, [_i32, ctypes.c_int64, _i32, _i32, _vp, _u64, _vp, _P(ctypes.c_double)]),
    "mgb_svd_workspace_size": (_i32, [_i32, ctypes.c_int64, ctypes.c_int64, _P(_u64)]),
    "mgb_svd": (_i32, [_i32, ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int64, _vp, _vp, _vp, _i32, _i32, _vp,
                       _u64, _vp]),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return os.environ.get("MUSCLE_GB300_LIB", LIB_PATH)


def load(build_if_missing: bool = True):
    """Returns the loaded library, building it in-tree when it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"libmuscle_gb300.so not found at {path}")
            from ._build import build

            build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)  # AttributeError when a declared symbol is missing
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class MuscleError(RuntimeError):
    """Base class of errors reported by the library."""


class ArgumentError(MuscleError, ValueError):
    """Julia's ArgumentError (src/Operations/binary_einsum.jl:54,82-83)."""


class DimensionMismatch(MuscleError, ValueError):
    """Julia's DimensionMismatch (src/Tensor.jl:23)."""


class UnsupportedError(ArgumentError):
    """A label pattern or element type the chosen form does not implement."""


class DeviceTimeout(MuscleError):
    """A bounded device-side wait gave up."""


class OutOfBudget(MuscleError, MemoryError):
    """The serving admission budget (bytes) is exhausted."""


_ERRORS = {
    ERR_ARGUMENT: ArgumentError,
    ERR_DIMENSION_MISMATCH: DimensionMismatch,
    ERR_UNSUPPORTED: UnsupportedError,
    ERR_WORKSPACE: MuscleError,
    ERR_CUDA: MuscleError,
    ERR_DEVICE_TIMEOUT: DeviceTimeout,
    ERR_OUT_OF_MEMORY: OutOfBudget,
    ERR_NOT_FINITE: ArgumentError,
}


def check(status: int, lib=None) -> None:
    if status == OK:
        return
    lib = lib or load()
    msg = (lib.mgb_last_error() or b"").decode(errors="replace")
    raise _ERRORS.get(status, MuscleError)(msg or f"libmuscle_gb300 status {status}")


def make_desc(dtype: int, modes, extents, strides):
    """Builds a TensorDesc; returns (desc, keepalive)."""
    r = len(modes)
    if r > MAX_RANK:
        raise ArgumentError(f"rank {r} exceeds {MAX_RANK}")
    m = (ctypes.c_int32 * max(r, 1))(*modes)
    e = (ctypes.c_int64 * max(r, 1))(*extents)
    s = (ctypes.c_int64 * max(r, 1))(*strides)
    d = TensorDesc(dtype, r, m, e, s)
    return d, (m, e, s)
