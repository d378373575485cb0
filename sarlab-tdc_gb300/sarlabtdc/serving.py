"""Request loop: continuous batching of focus jobs on one GPU (no reference counterpart).

``FocusServer`` wraps the engine's request loop (tdc_server_* of the C ABI): jobs
submitted from any thread are admitted by device-memory footprint, and every
focus launch carries work units of all admitted jobs, so a job that arrives
while others run starts in the next launch instead of waiting for them. A
job's image is bitwise the same alone and in any mix.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

import _tdc_capi as _lib


class FocusServer:
    def __init__(self, device: int = 0, memory_budget: int = 0, max_jobs: int = 32):
        h = C.c_void_p()
        _lib.check(_lib.lib().tdc_server_create(int(device), int(memory_budget), int(max_jobs), C.byref(h)))
        self._h = h
        self._keep = {}
        self._mu = threading.Lock()

    def submit(self, raw, sample_times, positions, grid, mod_rate, start_freq, velocity=None, attitude=None,
               boresight=(0.0, 1.0, 0.0), start=(0.0, float("inf"), False, False, True)) -> int:
        """Queue one focus job. ``positions`` [nPri, 3] (FP64 for double-float range/phase, or FP32),
        ``grid`` [..., 3] (FP32 or FP64). Returns the job id."""
        raw = np.ascontiguousarray(raw, dtype=np.complex64)
        n_pri, n_s = raw.shape
        st = np.ascontiguousarray(sample_times, dtype=np.float32)
        pos = np.ascontiguousarray(positions)
        pos64 = pos.astype(np.float64) if pos.dtype == np.float64 else None
        pos32 = None if pos64 is not None else pos.astype(np.float32)
        g = np.ascontiguousarray(np.asarray(grid).reshape(-1, 3))
        g64 = g if g.dtype == np.float64 else None
        g32 = None if g64 is not None else g.astype(np.float32)
        vel = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float32)
        att = None if attitude is None else np.ascontiguousarray(attitude, dtype=np.float32)
        image = np.zeros(g.shape[0], dtype=np.complex64)
        d = _lib.JobDesc()
        d.raw_iq, d.sample_times = raw.ctypes.data, st.ctypes.data
        d.position = None if pos32 is None else pos32.ctypes.data
        d.position_f64 = None if pos64 is None else pos64.ctypes.data
        d.velocity = None if vel is None else vel.ctypes.data
        d.attitude = None if att is None else att.ctypes.data
        d.n_pri, d.n_samples = n_pri, n_s
        d.mod_rate, d.start_freq = float(mod_rate), float(start_freq)
        d.body_boresight = (C.c_float * 3)(*boresight)
        d.grid = None if g32 is None else g32.ctypes.data
        d.grid_f64 = None if g64 is None else g64.ctypes.data
        d.n_pix = g.shape[0]
        c, b, cw, rw, tp = start
        d.doppler_win_center, d.doppler_bandwidth = float(c), float(b)
        d.dop_centroid_win, d.apply_range_win, d.doppler_win_taper = int(bool(cw)), int(bool(rw)), int(bool(tp))
        d.image = image.ctypes.data
        jid = C.c_uint64()
        with self._mu:
            _lib.check(_lib.lib().tdc_server_submit(self._h, C.byref(d), C.byref(jid)))
            self._keep[jid.value] = (raw, st, pos32, pos64, g32, g64, vel, att, image)
        return jid.value

    def wait(self, job_id: int, timeout_ms: int = -1):
        """(image complex64 [n_pix], info dict) once the job is done; raises on a job error."""
        info = _lib.JobInfo()
        rc = _lib.lib().tdc_server_wait(self._h, C.c_uint64(job_id), int(timeout_ms), C.byref(info))
        _lib.check(rc)
        with self._mu:
            keep = self._keep.pop(job_id)
        return keep[-1], info.as_dict()

    def stats(self) -> dict:
        s = _lib.ServerStats()
        _lib.check(_lib.lib().tdc_server_stats_get(self._h, C.byref(s)))
        return s.as_dict()

    def close(self):
        if self._h is not None and self._h.value:
            _lib.lib().tdc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
