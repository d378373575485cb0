"""ctypes binding of ``oracle/tdc_oracle.c`` -- TEST INFRASTRUCTURE ONLY.

Each function names the reference code it restates (paths relative to the
sarlab-tdc project). Inputs are numpy arrays; FP32 API inputs are widened to
FP64 exactly before the FP64 arithmetic, which is what "parity mode" means:
the oracle sees the same values the reference (and the GPU engine) receive.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from functools import lru_cache

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_lp = C.POINTER(C.c_long)


class _Problem(C.Structure):
    _fields_ = [
        ("n_pri", C.c_int),
        ("n_samples", C.c_int),
        ("raw", _fp),
        ("sample_times", _dp),
        ("pos", _dp), ("pos_cs", C.c_long), ("pos_ss", C.c_long),
        ("vel", _dp), ("vel_cs", C.c_long), ("vel_ss", C.c_long),
        ("att", _dp), ("att_cs", C.c_long), ("att_ss", C.c_long),
        ("mod_rate", C.c_double),
        ("start_freq", C.c_double),
        ("bore", C.c_double * 3),
        ("lambda_", C.c_double),
        ("grid", _dp),
        ("n_pix", C.c_long),
    ]


class _Opts(C.Structure):
    _fields_ = [
        ("dop_center", C.c_double),
        ("dop_bw", C.c_double),
        ("centroid_win", C.c_int),
        ("range_win", C.c_int),
        ("taper", C.c_int),
        ("skip_test", C.c_int),
        ("chunk", C.c_int),
        ("range_a", C.c_double),
        ("az_a", C.c_double),
    ]


@lru_cache(maxsize=1)
def lib() -> C.CDLL:
    path = _build.build_oracle()
    L = C.CDLL(str(path))
    L.tdco_focus.argtypes = [C.POINTER(_Problem), C.POINTER(_Opts), _lp, C.c_long, _dp, C.c_int]
    L.tdco_focus.restype = C.c_int
    L.tdco_adjoint_offsets.argtypes = [C.POINTER(_Problem), C.POINTER(_Opts), _dp, _lp, C.c_long, _dp, _dp,
                                       C.c_int]
    L.tdco_adjoint_offsets.restype = C.c_int
    L.tdco_range_window.argtypes = [_dp, C.c_int, C.c_int, C.c_double]
    L.tdco_range_window.restype = None
    L.tdco_wavelength_center.argtypes = [_fp, C.c_int, C.c_float, C.c_float]
    L.tdco_wavelength_center.restype = C.c_float
    L.tdco_window_is_nonzero.argtypes = [C.POINTER(_Problem), C.POINTER(_Opts), C.c_int, _dp]
    L.tdco_window_is_nonzero.restype = C.c_int
    L.tdco_skip_row_pri.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    L.tdco_skip_row_pri.restype = C.c_int
    L.tdco_skip_points.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.tdco_skip_points.restype = None
    for name in ("tdco_q_prod",):
        getattr(L, name).argtypes = [_dp, _dp, _dp]
        getattr(L, name).restype = None
    L.tdco_q_rot.argtypes = [_dp, _dp, _dp]
    L.tdco_q_rot.restype = None
    L.tdco_q_conj.argtypes = [_dp, _dp]
    L.tdco_q_conj.restype = None
    L.tdco_norm3.argtypes = [C.c_double] * 3
    L.tdco_norm3.restype = C.c_double
    L.tdco_dot3.argtypes = [_dp, _dp]
    L.tdco_dot3.restype = C.c_double
    L.tdco_doppler_centroid.argtypes = [_dp, _dp, C.c_double]
    L.tdco_doppler_centroid.restype = C.c_double
    L.tdco_doppler_freq.argtypes = [_dp, _dp, _dp, C.c_double]
    L.tdco_doppler_freq.restype = C.c_double
    L.tdco_doppler_window.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double]
    L.tdco_doppler_window.restype = C.c_double
    return L


@lru_cache(maxsize=1)
def refmath() -> C.CDLL | None:
    """The reference's own host-compiled gpumath.h / windowing.h, or None."""
    path = _build.build_refmath()
    if path is None or not os.path.exists(path):
        return None
    L = C.CDLL(str(path))
    L.ref_norm3.argtypes = [C.c_float] * 3
    L.ref_norm3.restype = C.c_float
    for name in ("ref_float2_add", "ref_float3_sub", "ref_q_prod", "ref_q_rot"):
        getattr(L, name).argtypes = [_fp, _fp, _fp]
        getattr(L, name).restype = None
    L.ref_q_conj.argtypes = [_fp, _fp]
    L.ref_q_conj.restype = None
    L.ref_dot3.argtypes = [_fp, _fp]
    L.ref_dot3.restype = C.c_float
    L.ref_doppler_centroid.argtypes = [_fp, _fp, C.c_float]
    L.ref_doppler_centroid.restype = C.c_float
    L.ref_doppler_freq.argtypes = [_fp, _fp, _fp, C.c_float]
    L.ref_doppler_freq.restype = C.c_float
    L.ref_doppler_window.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int]
    L.ref_doppler_window.restype = C.c_float
    for name in ("ref_range_window_a", "ref_azimuth_window_a"):
        getattr(L, name).argtypes = []
        getattr(L, name).restype = C.c_float
    L.ref_pri_chunksize.argtypes = []
    L.ref_pri_chunksize.restype = C.c_int
    return L


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _traj(arr, ncomp, n_pri, n_samples):
    """Normalise a trajectory array to FP64 with (chirp, sample) strides in elements.

    Accepts [n_pri, n_samples, ncomp] (per sample) or [n_pri, ncomp] (per chirp).
    """
    if arr is None:
        return None, 0, 0
    a = np.ascontiguousarray(np.asarray(arr), dtype=np.float64)
    if a.ndim == 3:
        assert a.shape == (n_pri, n_samples, ncomp), a.shape
        return a, n_samples * ncomp, ncomp
    if a.ndim == 2:
        assert a.shape == (n_pri, ncomp), a.shape
        return a, ncomp, 0
    raise ValueError("trajectory arrays are [nPri, nSamples, k] or [nPri, k]")


@dataclass
class Opts:
    """Arguments of TdcProcessor::start (tdcprocessor.h:67-68) plus compile-time constants."""
    dopplerWinCenter: float = 0.0
    dopplerBandwidth: float = float("inf")
    dopCentroidWin: bool = False
    applyRangeWin: bool = False
    dopplerWinTaper: bool = True
    skip_test: bool = True
    chunk: int = 128                     # PRI_CHUNKSIZE, tuning.h:18
    range_a: float = 25.0 / 46.0         # RANGE_WINDOW_A_PARAMETER, tuning.h:31
    az_a: float = 25.0 / 46.0            # AZIMUTH_WINDOW_A_PARAMETER, tuning.h:38

    def to_c(self) -> _Opts:
        # start() receives float arguments; widen the float value.
        return _Opts(float(np.float32(self.dopplerWinCenter)), float(np.float32(self.dopplerBandwidth)),
                     int(bool(self.dopCentroidWin)), int(bool(self.applyRangeWin)),
                     int(bool(self.dopplerWinTaper)), int(bool(self.skip_test)), int(self.chunk),
                     float(self.range_a), float(self.az_a))


@dataclass
class Problem:
    """One acquisition plus focus grid, as TdcProcessor::setRawData / setFocusGrid receive it.

    ``position`` may be FP32 per-sample [C, S, 3] (reference API) or FP64 per-chirp
    [C, 3]; ``grid`` is [..., 3] in FP32 or FP64. ``lam`` defaults to the
    reference's centre wavelength (tdcprocessor.cpp:204-208).
    """
    raw: np.ndarray
    sampleTimes: np.ndarray
    position: np.ndarray
    modRate: float
    startFreq: float
    grid: np.ndarray
    velocity: np.ndarray | None = None
    attitude: np.ndarray | None = None
    bodyBoresight: tuple = (0.0, 1.0, 0.0)
    lam: float | None = None
    _keep: list = field(default_factory=list, repr=False)

    def to_c(self) -> _Problem:
        raw = np.ascontiguousarray(self.raw, dtype=np.complex64)
        n_pri, n_samples = raw.shape
        rawf = raw.view(np.float32)
        st32 = np.ascontiguousarray(self.sampleTimes, dtype=np.float32)
        st = st32.astype(np.float64)
        pos, pcs, pss = _traj(self.position, 3, n_pri, n_samples)
        vel, vcs, vss = _traj(self.velocity, 3, n_pri, n_samples)
        att, acs, ass = _traj(self.attitude, 4, n_pri, n_samples)
        grid = np.ascontiguousarray(np.asarray(self.grid).reshape(-1, 3), dtype=np.float64)
        lam = self.lam
        if lam is None:
            lam = float(wavelength_center(st32, np.float32(self.modRate), np.float32(self.startFreq)))
        self._keep = [rawf, st, pos, vel, att, grid]
        p = _Problem()
        p.n_pri, p.n_samples = n_pri, n_samples
        p.raw = _ptr(rawf, C.c_float)
        p.sample_times = _ptr(st, C.c_double)
        p.pos, p.pos_cs, p.pos_ss = _ptr(pos, C.c_double), pcs, pss
        p.vel = _ptr(vel, C.c_double) if vel is not None else None
        p.vel_cs, p.vel_ss = vcs, vss
        p.att = _ptr(att, C.c_double) if att is not None else None
        p.att_cs, p.att_ss = acs, ass
        # setRawData takes float modRate / startFreq: widen those float values.
        p.mod_rate = float(np.float32(self.modRate))
        p.start_freq = float(np.float32(self.startFreq))
        p.bore = (C.c_double * 3)(*[float(np.float32(b)) for b in self.bodyBoresight])
        p.lambda_ = float(lam)
        p.grid = _ptr(grid, C.c_double)
        p.n_pix = grid.shape[0]
        return p


def _threads(n):
    return int(n) if n else (os.cpu_count() or 1)


def focus(problem: Problem, opts: Opts, pixels=None, threads=None) -> np.ndarray:
    """FP64 focused image (complex128) of all pixels, or of the flat pixel indices ``pixels``."""
    p = problem.to_c()
    o = opts.to_c()
    if pixels is None:
        n = p.n_pix
        idx = None
    else:
        idx = np.ascontiguousarray(pixels, dtype=np.int64)
        n = idx.size
    out = np.zeros(2 * n, dtype=np.float64)
    rc = lib().tdco_focus(C.byref(p), C.byref(o), _ptr(idx, C.c_long) if idx is not None else None, n,
                          _ptr(out, C.c_double), _threads(threads))
    if rc != 0:
        raise RuntimeError(f"tdco_focus failed ({rc})")
    return out.view(np.complex128)


def adjoint_offsets(problem: Problem, opts: Opts, offsets, grad_image, pixels=None, threads=None):
    """FP64 gradient [C, 3] of a real loss w.r.t. per-chirp position offsets.

    ``grad_image`` holds dL/dRe I + j dL/dIm I for each focused pixel.
    """
    p = problem.to_c()
    o = opts.to_c()
    g = np.ascontiguousarray(np.asarray(grad_image, dtype=np.complex128).ravel()).view(np.float64)
    if pixels is None:
        idx = None
        n = g.size // 2
    else:
        idx = np.ascontiguousarray(pixels, dtype=np.int64)
        n = idx.size
    off = None if offsets is None else np.ascontiguousarray(offsets, dtype=np.float64).reshape(-1, 3)
    grad = np.zeros((p.n_pri, 3), dtype=np.float64)
    rc = lib().tdco_adjoint_offsets(C.byref(p), C.byref(o), _ptr(off, C.c_double) if off is not None else None,
                                    _ptr(idx, C.c_long) if idx is not None else None, n,
                                    _ptr(g, C.c_double), _ptr(grad, C.c_double), _threads(threads))
    if rc != 0:
        raise RuntimeError(f"tdco_adjoint_offsets failed ({rc})")
    return grad


def range_window(n_samples: int, apply: bool = True, a: float = 25.0 / 46.0) -> np.ndarray:
    w = np.zeros(n_samples, dtype=np.float64)
    lib().tdco_range_window(_ptr(w, C.c_double), n_samples, int(apply), a)
    return w


def wavelength_center(sample_times, mod_rate, start_freq) -> np.float32:
    st = np.ascontiguousarray(sample_times, dtype=np.float32)
    return np.float32(lib().tdco_wavelength_center(_ptr(st, C.c_float), st.size, float(np.float32(mod_rate)),
                                                   float(np.float32(start_freq))))


def window_is_nonzero(problem: Problem, opts: Opts, chunk_idx: int, target) -> bool:
    p = problem.to_c()
    o = opts.to_c()
    t = np.ascontiguousarray(target, dtype=np.float64)
    return bool(lib().tdco_window_is_nonzero(C.byref(p), C.byref(o), chunk_idx, _ptr(t, C.c_double)))


def skip_row_pri(n_pri: int, chunk: int, chunk_idx: int, row: int) -> int:
    return int(lib().tdco_skip_row_pri(n_pri, chunk, chunk_idx, row))


def skip_points(n_samples: int, chunk: int = 128):
    rows = (C.c_int * 3)()
    samples = (C.c_int * 3)()
    lib().tdco_skip_points(n_samples, chunk, rows, samples)
    return list(rows), list(samples)
