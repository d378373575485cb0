"""ctypes binding of ``libtdc_gb300.so`` (the C ABI of ``include/tdc_gb300.h``).

The library is the only compute path: if it is missing, importing this module
raises ImportError (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("TDC_GB300_LIB", PKG_ROOT / "libtdc_gb300.so"))

TDC_OK = 0
TDC_ERR_INVALID_ARGUMENT = -1
TDC_ERR_CUDA = -2
TDC_ERR_STATE = -3
TDC_ERR_NO_MEMORY = -4
TDC_ERR_TIMEOUT = -5
TDC_ERR_UNSUPPORTED = -6
TDC_ERR_SHAPE = -7

PRECISION_FP32_BULK = 0
PRECISION_FP64_PHASE = 1

PATH_NAMES = {0: "fp32_bulk", 1: "fp64_phase", 2: "general", 3: "general_fp64", 4: "fp32_motion"}


class NoallocFocusArgs(C.Structure):
    """tdc_noalloc_focus_args of include/tdc_gb300.h."""
    _fields_ = [
        ("samples", C.c_void_p),
        ("chirps", C.c_void_p),
        ("skip_points", C.c_void_p),
        ("grid_hi", C.c_void_p),
        ("grid_lo", C.c_void_p),
        ("n_pix", C.c_int64),
        ("n_pri", C.c_int),
        ("n_samples", C.c_int),
        ("g0", C.c_double),
        ("g1", C.c_double),
        ("lambda_", C.c_float),
        ("doppler_bandwidth", C.c_float),
        ("doppler_win_taper", C.c_int),
    ]


NOALLOC_SCRATCH_BYTES = 32 << 20
NOALLOC_MAX_SAMPLES = 9104


class JobDesc(C.Structure):
    """tdc_job_desc of include/tdc_gb300.h."""
    _fields_ = [
        ("raw_iq", C.c_void_p),
        ("sample_times", C.c_void_p),
        ("position", C.c_void_p),
        ("position_f64", C.c_void_p),
        ("velocity", C.c_void_p),
        ("attitude", C.c_void_p),
        ("n_pri", C.c_int),
        ("n_samples", C.c_int),
        ("mod_rate", C.c_float),
        ("start_freq", C.c_float),
        ("body_boresight", C.c_float * 3),
        ("grid", C.c_void_p),
        ("grid_f64", C.c_void_p),
        ("n_pix", C.c_int64),
        ("doppler_win_center", C.c_float),
        ("doppler_bandwidth", C.c_float),
        ("dop_centroid_win", C.c_int),
        ("apply_range_win", C.c_int),
        ("doppler_win_taper", C.c_int),
        ("image", C.c_void_p),
    ]


class JobInfo(C.Structure):
    _fields_ = [
        ("submit_ms", C.c_double),
        ("admit_ms", C.c_double),
        ("first_launch_ms", C.c_double),
        ("done_ms", C.c_double),
        ("correlations", C.c_int64),
        ("status", C.c_int),
        ("path", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [
        ("jobs_submitted", C.c_int64),
        ("jobs_done", C.c_int64),
        ("jobs_failed", C.c_int64),
        ("launches", C.c_int64),
        ("correlations", C.c_int64),
        ("device_bytes_in_use", C.c_int64),
        ("queued", C.c_int),
        ("active", C.c_int),
        ("unbatched", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class StartStats(C.Structure):
    _fields_ = [
        ("h2d_ms", C.c_double),
        ("prep_ms", C.c_double),
        ("focus_ms", C.c_double),
        ("d2h_ms", C.c_double),
        ("total_ms", C.c_double),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("correlations", C.c_int64),
        ("path", C.c_int),
        ("kernel_launches", C.c_int),
        ("stage_samples", C.c_int),
        ("stage_chirps", C.c_int),
        ("general_variant", C.c_int),
        ("tile_cols", C.c_int),
        ("adjoint_stored", C.c_int),
        ("motion_segment", C.c_int),
        ("anchor_pixels", C.c_int),
        ("span_permille", C.c_int),
    ]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["path_name"] = PATH_NAMES.get(self.path, str(self.path))
        return d


_vp = C.c_void_p
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)

# (name, restype, argtypes) for every function of include/tdc_gb300.h.
SIGNATURES = [
    ("tdc_last_error", C.c_char_p, []),
    ("tdc_abi_version", C.c_int, []),
    ("tdc_processor_create", C.c_int, [C.c_int, C.POINTER(_vp)]),
    ("tdc_processor_destroy", C.c_int, [_vp]),
    ("tdc_processor_set_raw_data", C.c_int,
     [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_float, C.c_float, _vp]),
    ("tdc_processor_set_focus_grid", C.c_int, [_vp, _vp, C.c_int, C.c_int]),
    ("tdc_processor_start", C.c_int, [_vp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]),
    ("tdc_processor_image_buffer", _vp, [_vp]),
    ("tdc_processor_grid_shape", C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("tdc_processor_set_chirp_positions_f64", C.c_int, [_vp, _vp, C.c_int]),
    ("tdc_processor_set_focus_grid_f64", C.c_int, [_vp, _vp, C.c_int, C.c_int]),
    ("tdc_processor_set_precision", C.c_int, [_vp, C.c_int]),
    ("tdc_processor_set_trajectory_per_chirp", C.c_int, [_vp, _vp, _vp, _vp]),
    ("tdc_processor_last_stats", C.c_int, [_vp, C.POINTER(StartStats)]),
    ("tdc_range_window", C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    ("tdc_processor_set_skip_test", C.c_int, [_vp, C.c_int]),
    ("tdc_processor_set_motion_path", C.c_int, [_vp, C.c_int]),
    ("tdc_processor_set_anchored_ranges", C.c_int, [_vp, C.c_int]),
    ("tdc_processor_set_plan_pixels", C.c_int, [_vp, C.c_int64]),
    ("tdc_processor_prepare", C.c_int, [_vp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]),
    ("tdc_processor_upload_grid", C.c_int, [_vp]),
    ("tdc_processor_focus_device", C.c_int, [_vp, _vp, _vp]),
    ("tdc_processor_check", C.c_int, [_vp, _vp]),
    ("tdc_processor_num_pixels", C.c_int, [_vp, C.POINTER(C.c_int64)]),
    ("tdc_processor_path", C.c_int, [_vp]),
    ("tdc_processor_reads_host_memory", C.c_int, [_vp]),
    ("tdc_processor_set_image_output", C.c_int, [_vp, _vp, C.c_int64]),
    ("tdc_probe_fma", C.c_int, [C.c_int, C.c_int, C.c_int, _vp, C.POINTER(C.c_double), _vp]),
    ("tdc_selftest_wait_timeout", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    ("tdc_focus_noalloc", C.c_int, [C.POINTER(NoallocFocusArgs), _vp, _vp]),
    ("tdc_focus_noalloc_async", C.c_int, [C.POINTER(NoallocFocusArgs), _vp, _vp, _vp]),
    ("tdc_processor_set_chirp_offsets_device", C.c_int, [_vp, _vp, _vp]),
    ("tdc_processor_adjoint_device", C.c_int, [_vp, _vp, _vp, _vp]),
    ("tdc_processor_set_keep_chirp_sums", C.c_int, [_vp, C.c_int]),
    ("tdc_server_create", C.c_int, [C.c_int, C.c_size_t, C.c_int, C.POINTER(_vp)]),
    ("tdc_server_submit", C.c_int, [_vp, C.POINTER(JobDesc), C.POINTER(C.c_uint64)]),
    ("tdc_server_wait", C.c_int, [_vp, C.c_uint64, C.c_int, C.POINTER(JobInfo)]),
    ("tdc_server_stats_get", C.c_int, [_vp, C.POINTER(ServerStats)]),
    ("tdc_server_destroy", C.c_int, [_vp]),
]

_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is not built: the GB300 TDC engine has no CPU fallback; "
                "run `python -c 'import __graft_entry__ as g; g.build()'` first")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class TdcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


def last_error() -> str:
    return lib().tdc_last_error().decode(errors="replace")


def check(rc: int) -> None:
    """Raise the Python exception the reference's binding raises for this status."""
    if rc == TDC_OK:
        return
    msg = last_error()
    if rc == TDC_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)          # std::invalid_argument -> ValueError (pybind11)
    if rc == TDC_ERR_NO_MEMORY:
        raise MemoryError(msg)
    raise TdcError(rc, msg)            # std::runtime_error -> RuntimeError


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (or None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
