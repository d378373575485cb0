"""tdc_focus_noalloc: the focus entry point for callers that cannot allocate
device memory (fixed-budget real-time chains, plug-ins inside a framework that
owns the allocator, stream capture). Its scratch is a fixed array inside the
library, so it must give the same image as tdc_processor_focus_device, call
after call, with inputs the caller lays out itself as the header documents.

This file is collected last on purpose (test_zz_*), so a stop-at-first-failure
run has executed every other test before it."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tdc_testutil import max_phase_err, problem_from_api, rel_l2, run_engine

L2_TOL = 1e-4
PHASE_TOL = 1e-3
C0 = 299792458.0


def _affine_fit(sample_times, mod_rate, start_freq):
    """2 f_s / c = g0 + s g1, least squares on f_s = f0 + K t_s (the processor's fit)."""
    t = np.asarray(sample_times, np.float32).astype(np.float64)
    f = float(np.float32(start_freq)) + float(np.float32(mod_rate)) * t
    S = t.size
    if S == 1:
        return 2 * f[0] / C0, 0.0
    s = np.arange(S, dtype=np.float64)
    sm, fm = 0.5 * (S - 1), f.mean()
    F1 = np.sum((s - sm) * (f - fm)) / np.sum((s - sm) ** 2)
    F0 = fm - F1 * sm
    return 2 * F0 / C0, 2 * F1 / C0


def _device_inputs(api, grid, torch):
    """The documented device layout, built by the caller with its own memory."""
    raw = api["rawData"]
    n_pri, S = raw.shape
    s_pad = (S + 15) // 16 * 16
    samples = torch.zeros((n_pri, s_pad), dtype=torch.complex64, device="cuda")
    samples[:, :S] = torch.from_numpy(np.ascontiguousarray(raw)).cuda()
    rec = np.zeros((n_pri, 12), np.float32)
    rec[:, 0:3] = api["position"][:, 0, :]
    rec[:, 3] = 0.0                      # fixed Doppler window centre
    rec[:, 8:11] = api["velocity"][:, 0, :]
    chirps = torch.from_numpy(rec).cuda()
    g = np.asarray(grid, np.float32).reshape(-1, 3)
    gh = np.zeros((g.shape[0], 4), np.float32)
    gh[:, :3] = g
    grid_hi = torch.from_numpy(gh).cuda()
    st = api["sampleTimes"]
    chirp_t = float(np.float32(st[-1] - st[0]))
    f0 = float(np.float32(api["startFreq"]))
    centre = (f0 + (f0 + float(np.float32(api["modRate"])) * chirp_t)) / 2.0
    lam = float(np.float32(C0 / centre))
    g0, g1 = _affine_fit(st, api["modRate"], api["startFreq"])
    return samples, chirps, grid_hi, g0, g1, lam


@pytest.mark.gpu
def test_noalloc_focus_matches_device_focus_twice_in_a_row(cuda_device):
    import torch

    import _tdc_capi
    from sarlabtdc import scenes

    lib = _tdc_capi.lib()
    sc = scenes.small_scene(seed=61, n_pri=300, n_samples=100, nx=40, ny=30, device="cuda")
    api = sc.api_arrays()
    args = (0.0, float("inf"), False, False, True)
    _, stats, p = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "fp32_bulk"
    p.prepare(*args)
    p.uploadGrid()
    n_pix = p.numPixels()
    ref = torch.empty(n_pix, dtype=torch.complex64, device="cuda")
    p.focusDevice(ref)
    p.check()
    ref_np = ref.cpu().numpy()

    samples, chirps, grid_hi, g0, g1, lam = _device_inputs(api, sc.grid, torch)
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = samples.data_ptr()
    a.chirps = chirps.data_ptr()
    a.skip_points = None
    a.grid_hi = grid_hi.data_ptr()
    a.grid_lo = None
    a.n_pix = n_pix
    a.n_pri = sc.n_pri
    a.n_samples = sc.n_samples
    a.g0, a.g1 = g0, g1
    a.lambda_ = lam
    a.doppler_bandwidth = float("inf")
    a.doppler_win_taper = 1
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for _ in range(2):
        out = torch.full((n_pix,), complex(float("nan"), 0.0), dtype=torch.complex64, device="cuda")
        rc = lib.tdc_focus_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert rc == 0, _tdc_capi.last_error()
        outs.append(out.cpu().numpy())
    for o in outs:
        assert np.all(np.isfinite(o))
        assert rel_l2(o, ref_np) <= L2_TOL
        assert max_phase_err(o, ref_np) <= PHASE_TOL
    np.testing.assert_array_equal(outs[0], outs[1])


def _split(a):
    """Double-float pair (high, low) of an FP64 array as float32 arrays."""
    hi = np.asarray(a, np.float64).astype(np.float32)
    lo = (np.asarray(a, np.float64) - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def _skip_table(api, centre):
    """The documented skip-point layout, ceil(n_pri / 128) x 9 points x 8 floats (position xyz,
    window centre, velocity xyz, 0), at the reference's 3 x 3 (PRI, sample) points of each
    chunk -- stale staging rows of a partial last chunk included (tdcprocessor.cpp:347-383)."""
    n_pri, S = api["rawData"].shape
    chunk = 128
    rows, samples = oracle.skip_points(S, chunk)
    n_chunks = (n_pri + chunk - 1) // chunk
    tab = np.zeros((n_chunks, 9, 8), np.float32)
    for k in range(n_chunks):
        for i in range(3):
            pri = oracle.skip_row_pri(n_pri, chunk, k, rows[i])
            for j in range(3):
                tab[k, i * 3 + j, 3] = centre
                if pri >= 0:
                    tab[k, i * 3 + j, 0:3] = api["position"][pri, samples[j]]
                    tab[k, i * 3 + j, 4:7] = api["velocity"][pri, samples[j]]
    return tab


def _noalloc_args(api, grid, torch, pos64=None, grid64=None, centre=0.0, band=float("inf"), taper=True,
                  skip=False):
    """Arguments and caller-owned device buffers of one tdc_focus_noalloc call."""
    import _tdc_capi

    samples, chirps, grid_hi, g0, g1, lam = _device_inputs(api, grid, torch)
    rec = chirps.cpu().numpy()
    rec[:, 3] = np.float32(centre)
    keep = []
    if pos64 is not None:
        hi, lo = _split(pos64)
        rec[:, 0:3] = hi
        rec[:, 4:7] = lo
    chirps = torch.from_numpy(rec).cuda()
    grid_lo = None
    if grid64 is not None:
        hi, lo = _split(np.asarray(grid64).reshape(-1, 3))
        gh = np.zeros((hi.shape[0], 4), np.float32)
        gl = np.zeros((hi.shape[0], 4), np.float32)
        gh[:, :3], gl[:, :3] = hi, lo
        grid_hi = torch.from_numpy(gh).cuda()
        grid_lo = torch.from_numpy(gl).cuda()
    skip_dev = torch.from_numpy(_skip_table(api, np.float32(centre))).cuda() if skip else None
    keep += [samples, chirps, grid_hi, grid_lo, skip_dev]
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = samples.data_ptr()
    a.chirps = chirps.data_ptr()
    a.skip_points = None if skip_dev is None else skip_dev.data_ptr()
    a.grid_hi = grid_hi.data_ptr()
    a.grid_lo = None if grid_lo is None else grid_lo.data_ptr()
    a.n_pix = grid_hi.shape[0]
    a.n_pri, a.n_samples = api["rawData"].shape
    a.g0, a.g1 = g0, g1
    a.lambda_ = lam
    a.doppler_bandwidth = float(band)
    a.doppler_win_taper = int(bool(taper))
    return a, keep


def _noalloc_twice(a):
    """Two calls in a row (the shared scratch keeps the first call's contents)."""
    import torch

    import _tdc_capi

    lib = _tdc_capi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for _ in range(2):
        out = torch.full((a.n_pix,), complex(float("nan"), 0.0), dtype=torch.complex64, device="cuda")
        rc = lib.tdc_focus_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert rc == 0, _tdc_capi.last_error()
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    return outs[0]


@pytest.mark.gpu
def test_noalloc_plain_against_the_oracle(cuda_device):
    import torch

    from sarlabtdc import scenes

    sc = scenes.small_scene(seed=63, n_pri=300, n_samples=100, nx=40, ny=30, device="cuda")
    api = sc.api_arrays()
    a, keep = _noalloc_args(api, sc.grid, torch)
    got = _noalloc_twice(a)
    ref = oracle.focus(problem_from_api(api, sc.grid), oracle.Opts(applyRangeWin=False))
    assert rel_l2(got, ref) <= L2_TOL
    assert max_phase_err(got, ref) <= PHASE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("taper", [True, False])
def test_noalloc_finite_band_and_skip_points_against_the_oracle(cuda_device, taper):
    """Finite Doppler band (the instance that skips zero-window chirps) with the chunk skip
    test from a caller-built skip table; 750 chirps, so the last chunk is partial and its
    skip points read stale staging rows. The antenna moves along the rail, so the window
    and the skip test cut real work."""
    import torch

    from sarlabtdc import scenes

    sc = scenes.small_scene(seed=64, n_pri=750, n_samples=64, nx=21, ny=17, rail_len=0.75, device="cuda")
    api = sc.api_arrays()
    vel = np.zeros_like(api["velocity"])
    vel[..., 0] = 0.2
    api["velocity"] = vel
    centre, band = 2.0, 18.0
    a, keep = _noalloc_args(api, sc.grid, torch, centre=centre, band=band, taper=taper, skip=True)
    got = _noalloc_twice(a)
    prob = problem_from_api(api, sc.grid)
    ref = oracle.focus(prob, oracle.Opts(dopplerWinCenter=centre, dopplerBandwidth=band, applyRangeWin=False,
                                         dopplerWinTaper=taper, skip_test=True))
    full = oracle.focus(prob, oracle.Opts(applyRangeWin=False, dopplerWinTaper=taper))
    assert rel_l2(ref, full) > 0.05                      # the window does cut pixels' chirps
    no_skip = oracle.focus(prob, oracle.Opts(dopplerWinCenter=centre, dopplerBandwidth=band, applyRangeWin=False,
                                             dopplerWinTaper=taper, skip_test=False))
    assert rel_l2(ref, no_skip) > 0.05                   # and the skip test drops whole chunks
    # chirps at the inclusive band edge may fall either side in FP32: L2 bound only
    assert rel_l2(got, ref) <= 2e-4


@pytest.mark.gpu
def test_noalloc_double_float_positions_and_grid_against_the_oracle(cuda_device):
    """FP64 positions and grid passed as double-float pairs (low floats in the chirp records
    and grid_lo), against the oracle on the FP64 values."""
    import torch

    from sarlabtdc import scenes

    sc = scenes.small_scene(seed=65, n_pri=512, n_samples=256, nx=24, ny=24, jitter=0.5e-3, spacing=1e-3,
                            y0=0.6, rail_len=1.0, device="cuda")
    api = sc.api_arrays()
    a, keep = _noalloc_args(api, sc.grid, torch, pos64=sc.positions, grid64=sc.grid)
    got = _noalloc_twice(a)
    ref = oracle.focus(problem_from_api(api, sc.grid, pos64=sc.positions, grid64=True),
                       oracle.Opts(applyRangeWin=False))
    assert rel_l2(got, ref) <= L2_TOL
    assert max_phase_err(got, ref) <= PHASE_TOL
    # the low floats matter at this precision: the FP32-rounded inputs give a different image
    a32, keep32 = _noalloc_args(api, sc.grid, torch)
    assert rel_l2(_noalloc_twice(a32), ref) > rel_l2(got, ref)


def test_noalloc_rejects_rows_longer_than_its_stages():
    """Size check only: rows above TDC_NOALLOC_MAX_SAMPLES return TDC_ERR_UNSUPPORTED before
    any CUDA call (run where no GPU is present)."""
    import torch

    import _tdc_capi

    if torch.cuda.is_available():
        pytest.skip("host-side rejection is checked where no GPU is present")
    lib = _tdc_capi.lib()
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = a.chirps = a.grid_hi = 4096      # never dereferenced: rejected on size first
    a.n_pix = 512
    a.n_pri = 128
    a.n_samples = _tdc_capi.NOALLOC_MAX_SAMPLES + 1
    a.lambda_ = 0.0039
    a.doppler_bandwidth = float("inf")
    rc = lib.tdc_focus_noalloc(C.byref(a), C.c_void_p(4096), None)
    assert rc == _tdc_capi.TDC_ERR_UNSUPPORTED
    assert "nSamples" in _tdc_capi.last_error()


@pytest.mark.gpu
def test_noalloc_async_captured_in_a_cuda_graph(cuda_device):
    """tdc_focus_noalloc_async captured into a CUDA graph: a replay gives the blocking
    call's image bit for bit, and a replay after the caller rewrites the inputs in place
    focuses the new data (samples doubled: image exactly doubled); the status word the
    graph copies out reads 0."""
    import torch

    import _tdc_capi
    from sarlabtdc import scenes

    lib = _tdc_capi.lib()
    sc = scenes.small_scene(seed=62, n_pri=256, n_samples=128, nx=40, ny=30, device="cuda")
    api = sc.api_arrays()
    samples, chirps, grid_hi, g0, g1, lam = _device_inputs(api, sc.grid, torch)
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = samples.data_ptr()
    a.chirps = chirps.data_ptr()
    a.skip_points = None
    a.grid_hi = grid_hi.data_ptr()
    a.grid_lo = None
    a.n_pix = grid_hi.shape[0]
    a.n_pri = sc.n_pri
    a.n_samples = sc.n_samples
    a.g0, a.g1 = g0, g1
    a.lambda_ = lam
    a.doppler_bandwidth = float("inf")
    a.doppler_win_taper = 1
    n_pix = grid_hi.shape[0]
    ref = torch.empty(n_pix, dtype=torch.complex64, device="cuda")
    # the first call on the device (scratch address look-up) runs before any capture
    rc = lib.tdc_focus_noalloc(C.byref(a), C.c_void_p(ref.data_ptr()),
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _tdc_capi.last_error()
    ref_np = ref.cpu().numpy()
    assert np.all(np.isfinite(ref_np)) and np.abs(ref_np).max() > 0

    out = torch.full((n_pix,), complex(float("nan"), 0.0), dtype=torch.complex64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rc = lib.tdc_focus_noalloc_async(C.byref(a), C.c_void_p(out.data_ptr()), C.c_void_p(status.data_ptr()),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _tdc_capi.last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), ref_np)

    samples.mul_(2.0)
    status.fill_(-1)
    out.fill_(complex(float("nan"), 0.0))
    graph.replay()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    np.testing.assert_array_equal(out.cpu().numpy(), 2 * ref_np)


def test_noalloc_async_rejects_a_missing_status_word():
    """Argument check only: returns before any CUDA call."""
    import _tdc_capi

    lib = _tdc_capi.lib()
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = a.chirps = a.grid_hi = 4096      # never dereferenced
    a.n_pix = 512
    a.n_pri = 128
    a.n_samples = 256
    a.lambda_ = 0.0039
    a.doppler_bandwidth = float("inf")
    rc = lib.tdc_focus_noalloc_async(C.byref(a), C.c_void_p(4096), None, None)
    assert rc == _tdc_capi.TDC_ERR_INVALID_ARGUMENT
    assert "status word" in _tdc_capi.last_error()


def test_noalloc_rejects_grids_beyond_its_fixed_scratch():
    """Size check only: returns before any CUDA call (run where no GPU is present)."""
    import torch

    import _tdc_capi

    if torch.cuda.is_available():
        pytest.skip("host-side rejection is checked where no GPU is present")
    lib = _tdc_capi.lib()
    a = _tdc_capi.NoallocFocusArgs()
    a.samples = a.chirps = a.grid_hi = 4096      # never dereferenced: rejected on size first
    a.n_pix = (_tdc_capi.NOALLOC_SCRATCH_BYTES // 16) + 1
    a.n_pri = 128
    a.n_samples = 256
    a.lambda_ = 0.0039
    a.doppler_bandwidth = float("inf")
    rc = lib.tdc_focus_noalloc(C.byref(a), C.c_void_p(4096), None)
    assert rc == _tdc_capi.TDC_ERR_UNSUPPORTED
    assert "bytes of scratch" in _tdc_capi.last_error()
