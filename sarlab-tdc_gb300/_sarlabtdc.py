"""``_sarlabtdc`` -- the GB300 engine behind the reference's Python module interface.

Mirrors the pybind11 module of py-sarlabtdc (py-sarlabtdc/src/interface.cpp:9-22,
py-sarlabtdc/src/tdcprocessor_wrapper.cpp:19-170): class ``TdcProcessor(gpuNum)``
with ``setRawData``, ``setFocusGrid``, ``start`` and ``getFocusedImage``, the same
positional arguments, the same numpy conversions (any numeric array is cast to
C-contiguous complex64 / float32, like ``py::array_t<T, c_style>``), the same
shape checks and messages (RuntimeError), ValueError for ``nPri``/``nSamples`` <= 0,
and references kept to the arrays until they are replaced (the processor
borrows their memory, tdcprocessor.cpp:176-186). The calls go through the C ABI
of ``libtdc_gb300.so``; everything else in this class is additive.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

import _tdc_capi as _lib

__doc__ = "Time-domain correlation SAR processor for high bandwidth mmWave radars."


def _arr(x, dtype):
    return np.ascontiguousarray(np.asarray(x).astype(dtype, copy=False))


_TYPESTR = {"complex64": ("<c8", 8), "float64": ("<f8", 8)}


def _device_buffer(obj, dtype: str, n_elems: int, what: str) -> int:
    """Device address of a CUDA buffer holding at least n_elems contiguous elements of dtype:
    a torch tensor, any object with __cuda_array_interface__ (CuPy, Numba, ...), or a raw
    address (int, taken as is). Undersized, strided or mistyped buffers are refused, since
    the kernels write n_elems elements."""
    if isinstance(obj, int):
        return obj
    typestr, size = _TYPESTR[dtype]
    if hasattr(obj, "data_ptr") and hasattr(obj, "is_cuda"):  # torch
        import torch

        want = {"complex64": torch.complex64, "float64": torch.float64}[dtype]
        if not obj.is_cuda or obj.dtype != want or not obj.is_contiguous() or obj.numel() < n_elems:
            raise ValueError(f"{what} must be a contiguous CUDA {dtype} tensor of at least {n_elems} elements")
        return obj.data_ptr()
    cai = getattr(obj, "__cuda_array_interface__", None)
    if cai is None:
        raise ValueError(f"{what} must be a CUDA array (torch tensor or __cuda_array_interface__) or an address")
    count = int(np.prod(cai["shape"])) if cai["shape"] else 1
    contiguous = cai.get("strides") is None or cai["strides"] == tuple(
        int(np.prod(cai["shape"][i + 1:])) * size for i in range(len(cai["shape"])))
    if cai["typestr"] != typestr or not contiguous or count < n_elems:
        raise ValueError(f"{what} must be a contiguous {dtype} CUDA array of at least {n_elems} elements")
    return int(cai["data"][0])


def _check_image_array(out, rows, cols):
    if not isinstance(out, np.ndarray) or out.dtype != np.complex64 or out.shape != (rows, cols) \
            or not out.flags.c_contiguous or not out.flags.writeable:
        raise ValueError(f"out must be a writeable C-contiguous complex64 array of shape ({rows}, {cols})")


class TdcProcessor:
    """Time-domain correlation SAR processor (tdc-lib/include/tdcprocessor.h:42-200)."""

    def __init__(self, gpuNum: int):
        L = _lib.lib()
        h = C.c_void_p()
        _lib.check(L.tdc_processor_create(int(gpuNum), C.byref(h)))
        self._h = h
        self._raw_refs = ()
        self._grid_ref = None
        self._pos64_ref = None
        self._grid_rows = 0
        self._grid_cols = 0
        self._image_out = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().tdc_processor_destroy(h)
            except Exception:
                pass
            self._h = None

    # ---- reference methods -------------------------------------------------

    def start(self, dopplerWinCenter, dopplerBandwidth, dopCentroidWin, applyRangeWin, dopplerWinTaper=True):
        """Run the focus (tdcprocessor.h:67-68). Blocks until the image is on the host."""
        _lib.check(_lib.lib().tdc_processor_start(self._h, float(dopplerWinCenter), float(dopplerBandwidth),
                                                  int(bool(dopCentroidWin)), int(bool(applyRangeWin)),
                                                  int(bool(dopplerWinTaper))))

    def setRawData(self, rawData, priTimes, sampleTimes, position, velocity, attitude, modRate, startFreq,
                   bodyBoresight, /):
        """tdcprocessor_wrapper.cpp:27-126: ndim checks, then shape checks, then setRawData."""
        raw = _arr(rawData, np.complex64)
        pri = _arr(priTimes, np.float32)
        st = _arr(sampleTimes, np.float32)
        pos = _arr(position, np.float32)
        vel = _arr(velocity, np.float32)
        att = _arr(attitude, np.float32)
        bore = _arr(bodyBoresight, np.float32)
        if raw.ndim != 2:
            raise RuntimeError("rawData must be 2D")
        if pri.ndim != 1:
            raise RuntimeError("priTimes must be 1D")
        if st.ndim != 1:
            raise RuntimeError("sampleTimes must be 1D")
        if pos.ndim != 3:
            raise RuntimeError("position must be 3D")
        if vel.ndim != 3:
            raise RuntimeError("velocity must be 3D")
        if att.ndim != 3:
            raise RuntimeError("attitude must be 3D")
        if bore.ndim != 1:
            raise RuntimeError("bodyBoresight must be 1D")
        n_pri, n_samples = raw.shape
        if pri.shape[0] != n_pri:
            raise RuntimeError("priTimes shape is incorrect")
        if st.shape[0] != n_samples:
            raise RuntimeError("sampleTimes shape is incorrect")
        if pos.shape != (n_pri, n_samples, 3):
            raise RuntimeError("position shape is incorrect")
        if vel.shape != (n_pri, n_samples, 3):
            raise RuntimeError("velocity shape is incorrect")
        if att.shape != (n_pri, n_samples, 4):
            raise RuntimeError("attitude shape is incorrect")
        if bore.shape[0] != 3:
            raise RuntimeError("bodyBoresight shape is incorrect")
        self._raw_refs = (raw, pri, st, pos, vel, att, bore)
        self._pos64_ref = None
        p = _lib.ptr
        _lib.check(_lib.lib().tdc_processor_set_raw_data(
            self._h, p(raw), p(pri), p(st), p(pos), p(vel), p(att), int(n_pri), int(n_samples),
            float(modRate), float(startFreq), p(bore)))

    def setFocusGrid(self, focusGrid, /):
        """tdcprocessor_wrapper.cpp:129-153."""
        grid = _arr(focusGrid, np.float32)
        if grid.ndim != 3:
            raise RuntimeError("focusGrid must be 3D")
        rows, cols = grid.shape[0], grid.shape[1]
        if grid.shape[2] != 3:
            raise RuntimeError("focusGrid shape is incorrect")
        self._grid_ref = grid
        self._grid_rows, self._grid_cols = rows, cols
        _lib.check(_lib.lib().tdc_processor_set_focus_grid(self._h, _lib.ptr(grid), int(rows), int(cols)))

    def getFocusedImage(self, out=None):
        """tdcprocessor_wrapper.cpp:155-163: a new complex64 [rows, cols] copy of the image.

        Extension: ``out`` (a C-contiguous complex64 [rows, cols] array) receives the copy
        instead of a new array; the array given to setImageOutput is returned as it is."""
        rows, cols = self._grid_rows, self._grid_cols
        addr = _lib.lib().tdc_processor_image_buffer(self._h)
        if out is None:
            out = np.empty((rows, cols), dtype=np.complex64)
        else:
            _check_image_array(out, rows, cols)
        if addr and rows * cols:
            if addr != out.ctypes.data:
                C.memmove(out.ctypes.data, addr, rows * cols * 8)
        elif rows * cols:
            out[...] = 0  # the reference copies from a buffer that does not exist yet; we return zeros
        return out

    # ---- extensions (no reference counterpart) ------------------------------

    def setChirpPositionsF64(self, position):
        """Per-chirp FP64 antenna positions [nPri, 3] used for range and phase."""
        pos = np.ascontiguousarray(np.asarray(position, dtype=np.float64))
        if pos.ndim != 2 or pos.shape[1] != 3:
            raise RuntimeError("position shape is incorrect")
        self._pos64_ref = pos
        _lib.check(_lib.lib().tdc_processor_set_chirp_positions_f64(self._h, _lib.ptr(pos), int(pos.shape[0])))

    def setTrajectoryPerChirp(self, position, velocity=None, attitude=None):
        """Per-chirp trajectory [nPri, 3] / [nPri, 3] / [nPri, 4] (FP32) replacing setRawData's
        per-sample arrays; velocity and attitude default to zero and identity."""
        pos = _arr(position, np.float32)
        vel = None if velocity is None else _arr(velocity, np.float32)
        att = None if attitude is None else _arr(attitude, np.float32)
        n = self.numChirps()
        if pos.shape != (n, 3) or (vel is not None and vel.shape != (n, 3)) or \
                (att is not None and att.shape != (n, 4)):
            raise RuntimeError("trajectory shape is incorrect")
        self._traj_refs = (pos, vel, att)
        _lib.check(_lib.lib().tdc_processor_set_trajectory_per_chirp(self._h, _lib.ptr(pos), _lib.ptr(vel),
                                                                     _lib.ptr(att)))

    def setFocusGridF64(self, focusGrid):
        grid = np.ascontiguousarray(np.asarray(focusGrid, dtype=np.float64))
        if grid.ndim != 3:
            raise RuntimeError("focusGrid must be 3D")
        if grid.shape[2] != 3:
            raise RuntimeError("focusGrid shape is incorrect")
        self._grid_ref = grid
        self._grid_rows, self._grid_cols = grid.shape[0], grid.shape[1]
        _lib.check(_lib.lib().tdc_processor_set_focus_grid_f64(self._h, _lib.ptr(grid), int(grid.shape[0]),
                                                               int(grid.shape[1])))

    def setPrecision(self, precision: str):
        """'fp32' (double-float range/phase, FP32 bulk; default) or 'fp64' (plain FP64-phase comparator)."""
        code = {"fp32": _lib.PRECISION_FP32_BULK, "fp64": _lib.PRECISION_FP64_PHASE}[precision]
        _lib.check(_lib.lib().tdc_processor_set_precision(self._h, code))

    def setPlanPixels(self, n_pix: int):
        """Extension: plan the chirp groups as for a grid of n_pix pixels (0: the grid's own), so
        a row block of a larger grid focuses bit for bit like that grid (pixel sharding)."""
        _lib.check(_lib.lib().tdc_processor_set_plan_pixels(self._h, int(n_pix)))

    def setMotionPath(self, enable: bool):
        """Extension: per-sample positions that move smoothly within each chirp take the
        smooth-motion kernel (default) or, when off, the FP32 general kernel."""
        _lib.check(_lib.lib().tdc_processor_set_motion_path(self._h, int(bool(enable))))

    def setAnchoredRanges(self, enable: bool):
        """Extension: with an unbounded Doppler band, groups of consecutive pixels share a
        double-float anchor range per chirp and add their FP32 range differences (default on;
        taken when every pixel lies within 5 cm of its anchor). Off: every (pixel, chirp)
        range in double-float."""
        _lib.check(_lib.lib().tdc_processor_set_anchored_ranges(self._h, int(bool(enable))))

    def setSkipTest(self, enable: bool):
        _lib.check(_lib.lib().tdc_processor_set_skip_test(self._h, int(bool(enable))))

    def lastStats(self) -> dict:
        s = _lib.StartStats()
        _lib.check(_lib.lib().tdc_processor_last_stats(self._h, C.byref(s)))
        return s.as_dict()

    # device-resident use (torch tensors or raw device addresses)
    def prepare(self, dopplerWinCenter, dopplerBandwidth, dopCentroidWin, applyRangeWin, dopplerWinTaper=True):
        _lib.check(_lib.lib().tdc_processor_prepare(self._h, float(dopplerWinCenter), float(dopplerBandwidth),
                                                    int(bool(dopCentroidWin)), int(bool(applyRangeWin)),
                                                    int(bool(dopplerWinTaper))))

    def uploadGrid(self):
        _lib.check(_lib.lib().tdc_processor_upload_grid(self._h))

    def numChirps(self) -> int:
        return int(self._raw_refs[0].shape[0]) if self._raw_refs else 0

    def numPixels(self) -> int:
        n = C.c_int64()
        _lib.check(_lib.lib().tdc_processor_num_pixels(self._h, C.byref(n)))
        return n.value

    def setImageOutput(self, image):
        """Caller-owned image output: later start() calls write the image straight into
        ``image`` (a C-contiguous complex64 host array -- numpy, a CPU torch tensor, or any
        __array_interface__ object -- of at least rows x cols elements for the grid set at
        start), in place from the GPU where it reads and writes host memory coherently, else
        by one copy. ``None`` returns to the processor's own buffer. The array is kept alive
        here."""
        if image is None:
            _lib.check(_lib.lib().tdc_processor_set_image_output(self._h, None, 0))
            self._image_out = None
            return
        # numpy arrays, CPU torch tensors (pinned or not) and other __array_interface__ objects
        # are taken as views of their own memory
        arr = image if isinstance(image, np.ndarray) else np.asarray(image)
        if arr.dtype != np.complex64 or not arr.flags.c_contiguous or not arr.flags.writeable:
            raise ValueError("image output must be a writeable C-contiguous complex64 host array")
        _lib.check(_lib.lib().tdc_processor_set_image_output(self._h, arr.ctypes.data, int(arr.size) * 2))
        self._image_out = (image, arr)

    def readsHostMemory(self) -> bool:
        """True when the kernels read the input arrays in place over a coherent host link."""
        return bool(_lib.lib().tdc_processor_reads_host_memory(self._h))

    def path(self) -> str:
        return _lib.PATH_NAMES.get(_lib.lib().tdc_processor_path(self._h), "none")

    @staticmethod
    def _stream(stream):
        """A CUDA stream handle: an int, a torch stream, or None for torch's current stream."""
        if stream is None:
            import torch

            stream = torch.cuda.current_stream()
        return stream if isinstance(stream, int) else stream.cuda_stream

    def focusDevice(self, image, stream=None):
        """Focus the resident acquisition onto the resident grid into ``image``
        (complex64, numPixels() elements: a CUDA tensor, any __cuda_array_interface__ array,
        or a device address), asynchronously on ``stream`` (default: torch's current stream)."""
        addr = _device_buffer(image, "complex64", self.numPixels(), "image")
        _lib.check(_lib.lib().tdc_processor_focus_device(self._h, addr, self._stream(stream)))

    def setChirpOffsetsDevice(self, offsets, stream=None):
        """Antenna positions := base + offsets (a CUDA float64 tensor [nPri, 3] or None)."""
        addr = None if offsets is None else _device_buffer(offsets, "float64", 3 * self.numChirps(), "offsets")
        _lib.check(_lib.lib().tdc_processor_set_chirp_offsets_device(self._h, addr, self._stream(stream)))

    def adjointDevice(self, grad_image, grad_offsets, stream=None):
        """grad_offsets [nPri, 3] float64 (CUDA) <- adjoint of focusDevice applied to grad_image
        (complex64 CUDA, dL/dRe I + j dL/dIm I). Blocking."""
        gi = _device_buffer(grad_image, "complex64", self.numPixels(), "grad_image")
        go = _device_buffer(grad_offsets, "float64", 3 * self.numChirps(), "grad_offsets")
        _lib.check(_lib.lib().tdc_processor_adjoint_device(self._h, gi, go, self._stream(stream)))

    def keepChirpSums(self, keep=True):
        """Let device-resident focuses keep their per-chirp sums for the next adjointDevice
        (which then does half the arithmetic); False frees them."""
        _lib.check(_lib.lib().tdc_processor_set_keep_chirp_sums(self._h, int(bool(keep))))

    def check(self, stream=None):
        """Synchronise ``stream`` and raise if a focus kernel reported an error."""
        _lib.check(_lib.lib().tdc_processor_check(self._h, self._stream(stream)))
