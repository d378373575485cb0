"""GPU parity tests: the engine (through the C ABI, via the reference-shaped
_sarlabtdc binding) against the FP64 oracle on the same inputs.

Tolerances: the engine's stated accuracy against the FP64 oracle is
relative L2 <= 1e-4 and max phase error <= 1e-3 rad over pixels within 40 dB of
the peak. Tests whose Doppler windows have chirps close to the inclusive band
edge (where FP32 and FP64 may take different sides) use only the L2 bound.
"""
import math

import numpy as np
import pytest

import oracle
from sarlabtdc import scenes
from tdc_testutil import max_phase_err, peak_err, problem_from_api, rel_l2, run_engine

pytestmark = pytest.mark.gpu

L2_TOL = 1e-4
PHASE_TOL = 1e-3
INF = float("inf")


def _oracle(api, grid, start_args, pos64=None, grid64=False, pixels=None, skip_test=True):
    c, b, cw, rw = start_args[:4]
    taper = start_args[4] if len(start_args) > 4 else True
    prob = problem_from_api(api, grid, pos64=pos64, grid64=grid64)
    o = oracle.Opts(dopplerWinCenter=c, dopplerBandwidth=b, dopCentroidWin=cw, applyRangeWin=rw,
                    dopplerWinTaper=taper, skip_test=skip_test)
    return oracle.focus(prob, o, pixels=pixels)


def _check(img, ref, l2=L2_TOL, phase=PHASE_TOL):
    e_l2 = rel_l2(img, ref)
    assert e_l2 <= l2, f"relative L2 {e_l2:.3e} > {l2:.1e}"
    if phase is not None:
        e_ph = max_phase_err(img, ref)
        assert e_ph <= phase, f"max phase error {e_ph:.3e} rad > {phase:.1e}"
    return e_l2


def test_smoke_all_zero_inputs_like_reference_test(cuda_device):
    """tdctest/tdctest.cpp:21-59: 20 x 20 grid, nPri = 750, nSamples = 1500, zeros everywhere,
    B = 5 Hz, centroid windowing, range window. Antenna on every pixel -> NaN Doppler -> zero window."""
    C, S = 750, 1500
    api = dict(rawData=np.zeros((C, S), np.complex64), priTimes=np.zeros(C, np.float32),
               sampleTimes=np.zeros(S, np.float32), position=np.zeros((C, S, 3), np.float32),
               velocity=np.zeros((C, S, 3), np.float32), attitude=np.zeros((C, S, 4), np.float32),
               modRate=1.0, startFreq=1.0, bodyBoresight=np.array([0, 1, 0], np.float32))
    grid = np.zeros((20, 20, 3), np.float32)
    img, stats, _ = run_engine(api, grid, (0.0, 5.0, True, True))
    assert img.shape == (20, 20) and img.dtype == np.complex64
    assert np.all(img == 0)
    assert stats["kernel_launches"] >= 4


def _scene_api(sc):
    a = sc.api_arrays()
    return a


@pytest.mark.parametrize("n_samples", [128, 1, 17, 33, 1500])
def test_parity_plain(cuda_device, n_samples):
    sc = scenes.small_scene(seed=n_samples, n_pri=160, n_samples=n_samples, nx=19, ny=13, device="cuda")
    api = _scene_api(sc)
    args = (0.0, INF, False, False, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "fp32_bulk"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref)


def test_parity_range_window_and_partial_tiles(cuda_device):
    sc = scenes.small_scene(seed=5, n_pri=300, n_samples=96, nx=33, ny=31, device="cuda")  # 1023 px
    api = _scene_api(sc)
    args = (0.0, INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref)
    # single pixel
    one = sc.grid[:1, :1]
    img1, _, _ = run_engine(api, one, args)
    _check(img1, ref[:1, :1], phase=None)
    np.testing.assert_allclose(img1[0, 0], img[0, 0], rtol=2e-6)


def _moving_api(sc, speed=0.05, yaw_sigma=0.02, seed=0):
    """Per-chirp-constant velocity along the rail and a per-chirp attitude (yaw) jitter."""
    rng = np.random.default_rng(seed)
    api = sc.api_arrays()
    C, S = sc.n_pri, sc.n_samples
    vel = np.zeros((C, S, 3), np.float32)
    vel[..., 0] = speed
    ang = rng.normal(0, yaw_sigma, C)
    att = np.zeros((C, S, 4), np.float32)
    att[..., 0] = np.cos(ang / 2)[:, None]
    att[..., 3] = np.sin(ang / 2)[:, None]
    api["velocity"] = vel
    api["attitude"] = att
    return api


@pytest.mark.parametrize("taper,centroid", [(True, True), (False, False), (True, False)])
def test_parity_doppler_window_and_skip_test(cuda_device, taper, centroid):
    """Finite Doppler band: per-chirp windows, tapered or rectangular, fixed centre or centroid,
    and the per-chunk skip test (nPri = 750: a partial last chunk with stale staging rows)."""
    sc = scenes.small_scene(seed=11, n_pri=750, n_samples=64, nx=21, ny=17, rail_len=0.75, device="cuda")
    api = _moving_api(sc)
    args = (2.0, 18.0, centroid, True, taper)
    img, stats, _ = run_engine(api, sc.grid, args)
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    # some pixels must actually be windowed / skipped for this to test anything
    full = _oracle(api, sc.grid, (0.0, INF, False, True, taper)).reshape(img.shape)
    assert rel_l2(ref, full) > 0.05
    _check(img, ref, l2=2e-4, phase=None)


def test_skip_test_can_be_disabled(cuda_device):
    sc = scenes.small_scene(seed=12, n_pri=384, n_samples=32, nx=16, ny=16, rail_len=0.5, device="cuda")
    api = _moving_api(sc, speed=0.08)
    args = (0.0, 12.0, False, True, False)
    img, _, _ = run_engine(api, sc.grid, args, skip_test=False)
    ref = _oracle(api, sc.grid, args, skip_test=False).reshape(img.shape)
    _check(img, ref, l2=2e-4, phase=None)
    img_skip, _, _ = run_engine(api, sc.grid, args, skip_test=True)
    ref_skip = _oracle(api, sc.grid, args, skip_test=True).reshape(img.shape)
    _check(img_skip, ref_skip, l2=2e-4, phase=None)


def test_parity_fp64_positions_and_grid(cuda_device):
    """Jittered FP64 trajectory and FP64 grid (the precision-study inputs)."""
    sc = scenes.small_scene(seed=21, n_pri=512, n_samples=256, nx=24, ny=24, jitter=0.5e-3, spacing=1e-3,
                            y0=0.6, rail_len=1.0, device="cuda")
    api = sc.api_arrays()
    args = (0.0, INF, False, False, True)
    img, stats, _ = run_engine(api, sc.grid, args, pos64=sc.positions, grid64=sc.grid)
    assert stats["path_name"] == "fp32_bulk"
    ref = _oracle(api, sc.grid, args, pos64=sc.positions, grid64=True).reshape(img.shape)
    _check(img, ref)
    assert peak_err(img, ref) < 1e-5


def test_fp64_phase_comparator(cuda_device):
    sc = scenes.small_scene(seed=22, n_pri=256, n_samples=128, nx=20, ny=20, jitter=0.3e-3, device="cuda")
    api = sc.api_arrays()
    args = (0.0, INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args, pos64=sc.positions, grid64=sc.grid, precision="fp64")
    assert stats["path_name"] == "fp64_phase"
    ref = _oracle(api, sc.grid, args, pos64=sc.positions, grid64=True).reshape(img.shape)
    _check(img, ref)


def test_general_path_per_sample_trajectory(cuda_device):
    """position[c, s] varies within the chirp (tdckernels.cu:204-208 reads it per element)."""
    sc = scenes.small_scene(seed=23, n_pri=192, n_samples=64, nx=14, ny=12, device="cuda")
    api = sc.api_arrays()
    C, S = sc.n_pri, sc.n_samples
    pos = api["position"].astype(np.float64)
    pos[..., 0] += (np.arange(S) / S * 0.4e-3)[None, :]       # antenna keeps moving during the chirp
    api["position"] = pos.astype(np.float32)
    api["velocity"] = np.zeros((C, S, 3), np.float32)
    api["velocity"][..., 0] = 0.02
    args = (0.0, 40.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "general"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref, l2=2e-4, phase=None)


def test_general_path_nonuniform_sample_times(cuda_device):
    sc = scenes.small_scene(seed=24, n_pri=128, n_samples=96, nx=12, ny=10, device="cuda")
    api = sc.api_arrays()
    rng = np.random.default_rng(3)
    st = api["sampleTimes"].astype(np.float64)
    st = st + rng.uniform(-0.3, 0.3, st.shape) * (st[1] - st[0])
    api["sampleTimes"] = st.astype(np.float32)
    args = (0.0, INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "general"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref)


def test_repeatable_and_linear(cuda_device):
    sc = scenes.small_scene(seed=31, n_pri=256, n_samples=64, nx=16, ny=16, device="cuda")
    api = sc.api_arrays()
    args = (0.0, INF, False, True, True)
    a, _, _ = run_engine(api, sc.grid, args)
    b, _, _ = run_engine(api, sc.grid, args)
    np.testing.assert_array_equal(a, b)
    api2 = dict(api)
    api2["rawData"] = (api["rawData"] * np.float32(2.0)).astype(np.complex64)
    c, _, _ = run_engine(api2, sc.grid, args)
    np.testing.assert_array_equal(c, 2 * a)          # scaling by 2 is exact through every FP32 step


def test_processor_reuse_and_reference_call_order(cuda_device):
    import _sarlabtdc

    sc = scenes.small_scene(seed=41, n_pri=128, n_samples=32, nx=8, ny=8, device="cuda")
    api = sc.api_arrays()
    p = _sarlabtdc.TdcProcessor(0)
    with pytest.raises(RuntimeError):
        p.start(0.0, INF, False, True)              # before setRawData / setFocusGrid
    p.setRawData(*api.values())
    with pytest.raises(RuntimeError):
        p.start(0.0, INF, False, True)
    p.setFocusGrid(sc.grid)
    p.start(0.0, INF, False, True)
    first = p.getFocusedImage()
    assert first.shape == (8, 8) and first.dtype == np.complex64
    first[...] = 0                                   # getFocusedImage returns a copy
    p.start(0.0, INF, False, True)
    again = p.getFocusedImage()
    assert np.abs(again).max() > 0
    smaller = sc.grid[:3, :5]
    p.setFocusGrid(smaller)
    p.start(0.0, INF, False, True)
    assert p.getFocusedImage().shape == (3, 5)
    np.testing.assert_array_equal(p.getFocusedImage(), again[:3, :5])
    with pytest.raises(ValueError):
        p.setRawData(np.zeros((0, 4), np.complex64), np.zeros(0, np.float32), np.zeros(4, np.float32),
                     np.zeros((0, 4, 3), np.float32), np.zeros((0, 4, 3), np.float32),
                     np.zeros((0, 4, 4), np.float32), 1.0, 1.0, np.zeros(3, np.float32))


def test_device_resident_focus_matches_start(cuda_device):
    import torch
    import _sarlabtdc

    sc = scenes.small_scene(seed=51, n_pri=256, n_samples=64, nx=20, ny=18, device="cuda")
    api = sc.api_arrays()
    args = (0.0, INF, False, True, True)
    img, _, p = run_engine(api, sc.grid, args)
    p.prepare(*args)
    p.uploadGrid()
    out = torch.empty(p.numPixels(), dtype=torch.complex64, device="cuda")
    p.focusDevice(out)
    p.check()
    np.testing.assert_array_equal(out.cpu().numpy().reshape(img.shape), img)
    # on a torch stream
    s = torch.cuda.Stream()
    out2 = torch.zeros_like(out)
    p.focusDevice(out2, stream=s)
    p.check(stream=s)
    np.testing.assert_array_equal(out2.cpu().numpy().reshape(img.shape), img)


def test_cpp_tdcprocessor_smoke(cuda_device, tmp_path):
    """The tdctest-shaped C++ program runs against the engine."""
    import subprocess

    from test_capi_cpu import _cpp_build

    r = subprocess.run([str(_cpp_build(tmp_path))], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_per_chirp_trajectory_matches_per_sample_arrays(cuda_device):
    """setTrajectoryPerChirp (ingest extension) gives the same image as the reference's per-sample arrays."""
    import _sarlabtdc

    sc = scenes.small_scene(seed=81, n_pri=300, n_samples=80, nx=20, ny=18, device="cuda")
    api = _moving_api(sc, speed=0.03)
    args = (1.0, 25.0, True, True, True)
    img, _, _ = run_engine(api, sc.grid, args)
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setTrajectoryPerChirp(api["position"][:, 0, :], api["velocity"][:, 0, :], api["attitude"][:, 0, :])
    p.setFocusGrid(sc.grid)
    p.start(*args)
    np.testing.assert_array_equal(p.getFocusedImage(), img)


def test_in_place_host_reads_match_staged_copies(cuda_device, monkeypatch):
    """Where the device reads pageable host memory coherently, the raw rows, trajectory scan
    and grid are read in place; the image must equal the staged-copy path bit for bit."""
    sc = scenes.small_scene(seed=91, n_pri=260, n_samples=72, nx=21, ny=19, jitter=0.1e-3, device="cuda")
    api = _moving_api(sc, speed=0.02)
    args = (0.0, 30.0, True, True, True)
    monkeypatch.setenv("TDC_GB300_HOST_READS", "0")
    staged, st_a, pa = run_engine(api, sc.grid, args)
    assert not pa.readsHostMemory()
    monkeypatch.delenv("TDC_GB300_HOST_READS")
    direct, st_b, pb = run_engine(api, sc.grid, args, pos64=sc.positions, grid64=None)
    print("device reads host memory in place:", pb.readsHostMemory())
    monkeypatch.setenv("TDC_GB300_HOST_READS", "0")
    staged64, _, _ = run_engine(api, sc.grid, args, pos64=sc.positions)
    monkeypatch.delenv("TDC_GB300_HOST_READS")
    direct32, _, _ = run_engine(api, sc.grid, args)
    np.testing.assert_array_equal(direct32, staged)
    np.testing.assert_array_equal(direct, staged64)
    # per-sample motion is detected the same way on both paths
    pos = api["position"].astype(np.float64)
    pos[..., 0] += (np.arange(sc.n_samples) / sc.n_samples * 0.2e-3)[None, :]
    api["position"] = pos.astype(np.float32)
    _, st_c, _ = run_engine(api, sc.grid, args)
    assert st_c["path_name"] == "general"


@pytest.mark.parametrize("host_reads", ["1", "0"])
def test_image_output_into_caller_buffer(cuda_device, monkeypatch, host_reads):
    """setImageOutput: start() writes into the caller's array (in place from the GPU where it
    reads and writes host memory, else by one copy); the image equals the default buffer's."""
    import _sarlabtdc

    if host_reads == "0":
        monkeypatch.setenv("TDC_GB300_HOST_READS", "0")
    sc = scenes.small_scene(seed=17, n_pri=200, n_samples=64, nx=23, ny=17, device="cuda")
    api = sc.api_arrays()
    args = (0.0, INF, False, True, True)
    ref, _, _ = run_engine(api, sc.grid, args)
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                 api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
    p.setFocusGrid(sc.grid)
    out = np.full(ref.shape, np.complex64(7 + 7j))
    p.setImageOutput(out)
    p.start(*args)
    np.testing.assert_array_equal(out, ref)
    st = p.lastStats()
    if p.readsHostMemory():
        assert st["d2h_bytes"] == 0
    else:
        assert st["d2h_bytes"] == ref.size * 8
    assert p.getFocusedImage() is not out and np.array_equal(p.getFocusedImage(), ref)
    again = np.empty_like(ref)
    assert p.getFocusedImage(out=again) is again and np.array_equal(again, ref)
    # a buffer smaller than the grid is refused at start(), before any write
    small = np.zeros((2, 2), np.complex64)
    p.setImageOutput(small)
    with pytest.raises(ValueError):
        p.start(*args)
    assert np.all(small == 0)
    p.setImageOutput(None)
    p.start(*args)
    np.testing.assert_array_equal(p.getFocusedImage(), ref)
    with pytest.raises(ValueError):
        p.setImageOutput(np.zeros((4, 4), np.complex128))
    # a pinned CPU torch tensor as the output (a view of its memory, no copy through numpy)
    import torch

    t = torch.zeros(ref.shape, dtype=torch.complex64).pin_memory()
    p.setImageOutput(t)
    p.start(*args)
    np.testing.assert_array_equal(t.numpy(), ref)


def _general_api(sc, traj=False, win=False, nonunif=False, drift=0.3e-3, seed=5):
    """Per-sample inputs: positions drifting within each chirp, per-sample velocity, jittered
    sample times (any combination)."""
    rng = np.random.default_rng(seed)
    api = sc.api_arrays()
    C, S = sc.n_pri, sc.n_samples
    if traj:
        pos = api["position"].astype(np.float64)
        pos += (np.arange(S) / S)[None, :, None] * rng.normal(0.0, drift, (C, 1, 3))
        api["position"] = pos.astype(np.float32)
    if win:
        vel = np.zeros((C, S, 3), np.float32)
        vel[..., 0] = 0.05 + 0.01 * np.sin(np.arange(S) / 7.0)[None, :]
        vel[..., 1] = 0.01 * rng.normal(size=(C, 1))
        api["velocity"] = vel
    if nonunif:
        st = api["sampleTimes"].astype(np.float64)
        st += rng.uniform(-0.3, 0.3, st.shape) * (st[1] - st[0])
        api["sampleTimes"] = st.astype(np.float32)
    return api


@pytest.mark.parametrize("case", ["traj", "traj_wide", "win", "traj_win", "nonunif", "traj_nonunif", "all"])
def test_fp32_general_kernel_variants(cuda_device, case):
    """FP32 general kernel (per-sample positions / windows, non-uniform sampling) against the
    FP64 oracle, which evaluates range, phase and window per element. traj_wide moves the
    antenna centimetres within a chirp (the longer range-change series, reduced phase)."""
    sc = scenes.small_scene(seed=31, n_pri=200, n_samples=80, nx=17, ny=13, device="cuda")
    traj = "traj" in case or case == "all"
    win = "win" in case or case == "all"
    nonunif = "nonunif" in case or case == "all"
    api = _general_api(sc, traj=traj, win=win, nonunif=nonunif, drift=3e-3 if case == "traj_wide" else 0.3e-3)
    args = (0.0, 30.0 if win else INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args, motion=False)
    assert stats["path_name"] == "general"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    if win:
        full = _oracle(api, sc.grid, (0.0, INF, False, True, True)).reshape(img.shape)
        assert rel_l2(ref, full) > 0.05  # the window must matter
        _check(img, ref, l2=2e-4, phase=None)
    else:
        _check(img, ref)


def test_general_inputs_fp64_precision_and_fallback(cuda_device):
    """FP64 precision on per-sample inputs takes the FP64 general kernel; intra-chirp motion
    too large for the FP32 range-change series falls back to it as well."""
    sc = scenes.small_scene(seed=32, n_pri=160, n_samples=64, nx=13, ny=11, device="cuda")
    api = _general_api(sc, traj=True, win=True)
    args = (0.0, 30.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args, precision="fp64")
    assert stats["path_name"] == "general_fp64"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref, l2=2e-4, phase=None)
    big = _general_api(sc, traj=True, drift=40e-3)     # centimetres within a chirp at ~0.3 m range
    img, stats, _ = run_engine(big, sc.grid, (0.0, INF, False, True, True))
    assert stats["path_name"] == "general_fp64"
    ref = _oracle(big, sc.grid, (0.0, INF, False, True, True)).reshape(img.shape)
    _check(img, ref)


def test_per_sample_motion_without_window_effect_takes_bulk_path(cuda_device):
    """Velocity varying within chirps cannot change an unbounded-band window: one record per
    chirp describes every sample and the FP32-bulk kernel runs."""
    sc = scenes.small_scene(seed=33, n_pri=150, n_samples=48, nx=12, ny=10, device="cuda")
    api = _general_api(sc, win=True)
    args = (0.0, INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "fp32_bulk"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref)


@pytest.mark.parametrize("n_samples,nx,ny", [(1, 7, 5), (17, 1, 1), (33, 23, 29), (1500, 9, 4)])
def test_fp32_general_kernel_odd_sizes(cuda_device, n_samples, nx, ny):
    """General kernel on ragged shapes: one sample, one pixel, partial tiles, long chirps
    (positions and windows per sample, jittered sample times)."""
    sc = scenes.small_scene(seed=51 + n_samples, n_pri=140, n_samples=n_samples, nx=nx, ny=ny, device="cuda")
    api = _general_api(sc, traj=True, win=True, nonunif=n_samples > 1)
    args = (0.0, 30.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    # one sample per chirp cannot vary within the chirp: the bulk kernel takes it
    assert stats["path_name"] == ("general" if n_samples > 1 else "fp32_bulk")
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref, l2=2e-4, phase=None)


def test_processors_on_concurrent_threads_match_sequential_runs(cuda_device):
    """Processors with different sample counts (different kernel launch shapes and shared-
    memory sizes) focusing at the same time from several host threads give the images they
    give one at a time."""
    import threading

    scs = [scenes.small_scene(seed=61 + k, n_pri=300 + 37 * k, n_samples=S, nx=30, ny=20, device="cuda")
           for k, S in enumerate((64, 200, 513, 1024))]
    args = (0.0, INF, False, True, True)
    alone = [run_engine(sc.api_arrays(), sc.grid, args)[0] for sc in scs]
    out = [None] * len(scs)
    errors = []

    def work(k):
        try:
            for _ in range(3):
                out[k] = run_engine(scs[k].api_arrays(), scs[k].grid, args)[0]
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    ths = [threading.Thread(target=work, args=(k,)) for k in range(len(scs))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    assert not errors, errors
    for a, b in zip(alone, out):
        np.testing.assert_array_equal(a, b)


def test_empty_grid_gives_an_empty_image(cuda_device):
    """A focus grid with no pixels: start() succeeds and the image is empty (the reference
    loops over zero pixels)."""
    sc = scenes.small_scene(seed=71, n_pri=64, n_samples=32, nx=4, ny=4, device="cuda")
    img, stats, _ = run_engine(sc.api_arrays(), np.zeros((0, 5, 3), np.float32), (0.0, INF, False, True, True))
    assert img.shape == (0, 5)
    assert stats["correlations"] == 0


@pytest.mark.parametrize("n_samples,band", [(9000, INF), (12000, 40.0), (20000, INF)])
def test_long_chirps_are_staged_in_segments(cuda_device, n_samples, band):
    """Rows longer than the bulk kernel's pipeline stages hold are staged in segments and
    stay on the FP32-bulk path (parity with the oracle; a finite band takes the
    zero-window-skipping instance)."""
    sc = scenes.small_scene(seed=81, n_pri=40, n_samples=n_samples, nx=10, ny=8, rail_len=0.1, device="cuda")
    api = _moving_api(sc, speed=0.05) if np.isfinite(band) else sc.api_arrays()
    args = (0.0, band, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "fp32_bulk"
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    _check(img, ref, l2=2e-4 if np.isfinite(band) else L2_TOL, phase=None if np.isfinite(band) else PHASE_TOL)


@pytest.mark.parametrize("case,n_samples", [("traj_win", 6000), ("traj", 9000), ("nonunif", 5000), ("all", 3000)])
def test_fp32_general_kernel_long_chirps_in_segments(cuda_device, case, n_samples):
    """Per-sample inputs with rows longer than the general kernel's stages: rows (and the
    per-sample frequency tables) are staged in segments, last segment first, with each
    chirp's Horner state carried across them; the FP32 general kernel keeps the job
    (parity with the FP64 oracle)."""
    sc = scenes.small_scene(seed=91, n_pri=36, n_samples=n_samples, nx=9, ny=7, rail_len=0.1, device="cuda")
    traj = "traj" in case or case == "all"
    win = "win" in case or case == "all"
    nonunif = "nonunif" in case or case == "all"
    api = _general_api(sc, traj=traj, win=win, nonunif=nonunif, drift=0.1e-3)
    args = (0.0, 30.0 if win else INF, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args, motion=False)
    assert stats["path_name"] == "general"
    assert 0 < stats["stage_samples"] < n_samples and stats["stage_chirps"] == 1
    assert stats["stage_samples"] % 16 == 0
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    if win:
        _check(img, ref, l2=2e-4, phase=None)
    else:
        _check(img, ref)


def test_fp32_general_kernel_stages_whole_rows_when_they_fit(cuda_device):
    """Short per-sample rows are staged whole, several chirps a stage."""
    sc = scenes.small_scene(seed=92, n_pri=64, n_samples=64, nx=8, ny=8, device="cuda")
    api = _general_api(sc, traj=True)
    img, stats, _ = run_engine(api, sc.grid, (0.0, INF, False, True, True), motion=False)
    assert stats["path_name"] == "general"
    assert stats["stage_samples"] == 64 and stats["stage_chirps"] > 1
    _check(img, _oracle(api, sc.grid, (0.0, INF, False, True, True)).reshape(img.shape))


@pytest.mark.parametrize("n_pri,n_samples,nx,ny", [(1, 1, 1, 1), (1, 64, 3, 5), (2, 3, 17, 31), (129, 17, 23, 23),
                                                   (127, 16, 32, 16), (257, 5, 1, 600)])
def test_parity_ragged_shapes(cuda_device, n_pri, n_samples, nx, ny):
    """Ragged acquisitions: one chirp, one sample, one pixel, chirp counts either side of
    the 128-chirp skip chunk, pixel counts either side of the 512-pixel tile; an unbounded
    band and a finite one (per-chirp windows, skip test on partial chunks) on the FP32-bulk
    kernel, and positions moving within the chirps on the smooth-motion kernel and on the
    FP32 general kernel."""
    sc = scenes.small_scene(seed=100 + n_pri + n_samples, n_pri=n_pri, n_samples=n_samples, nx=nx, ny=ny,
                            device="cuda")
    cases = [(_scene_api(sc), (0.0, INF, False, True, True), "fp32_bulk", True),
             (_moving_api(sc, speed=0.08), (2.0, 18.0, False, True, True), "fp32_bulk", True)]
    if n_samples > 1:
        cases.append((_general_api(sc, traj=True), (0.0, INF, False, True, True), "general", False))
    if n_samples > 2:
        # motion of a micrometre within the chirp: short rows with more motion change the phase
        # too fast along the chirp for the smooth-motion kernel's segments (the general kernel
        # takes them, as above)
        cases.append((_general_api(sc, traj=True, drift=1e-6), (0.0, INF, False, True, True), "fp32_motion", True))
    rng = np.random.default_rng(n_pri + n_samples)
    for api, args, path, motion in cases:
        if not np.any(api["rawData"]):
            # a one-sample chirp simulated under a Hann taper is all zero: use seeded noise
            raw = rng.normal(size=(n_pri, n_samples, 2)).astype(np.float32)
            api["rawData"] = np.ascontiguousarray(raw[..., 0] + 1j * raw[..., 1]).astype(np.complex64)
        img, stats, _ = run_engine(api, sc.grid, args, motion=motion)
        assert img.shape == (ny, nx)
        assert stats["path_name"] == path
        ref = _oracle(api, sc.grid, args).reshape(img.shape)
        assert np.all(np.isfinite(img))
        if not np.any(ref):
            assert not np.any(img)  # every chirp windowed out: the reference's image is all zero
        elif np.isfinite(args[1]):
            _check(img, ref, l2=2e-4, phase=None)
        else:
            _check(img, ref)


@pytest.mark.parametrize("general", [False, True])
def test_block_tiles_under_a_finite_band(cuda_device, general):
    """A finite Doppler band with the antenna moving along the grid's columns: the work
    tiles become blocks of 32 rows x 16 columns (ragged at the grid's edges: 40 x 35
    pixels); parity with the oracle on the bulk and the general kernel, and flat tiles
    again for an unbounded band."""
    sc = scenes.small_scene(seed=93, n_pri=400, n_samples=48, nx=40, ny=35, rail_len=0.4, device="cuda")
    api = _moving_api(sc, speed=0.08)
    if general:
        api = _general_api(sc, traj=True)
        api["velocity"] = _moving_api(sc, speed=0.08)["velocity"]
    args = (0.0, 14.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == ("general" if general else "fp32_bulk")
    assert stats["tile_cols"] == 16
    ref = _oracle(api, sc.grid, args).reshape(img.shape)
    full = _oracle(api, sc.grid, (0.0, INF, False, True, True)).reshape(img.shape)
    assert rel_l2(ref, full) > 0.05  # the band must zero part of the image
    _check(img, ref, l2=2e-4, phase=None)
    img_inf, stats_inf, _ = run_engine(api, sc.grid, (0.0, INF, False, True, True))
    assert stats_inf["tile_cols"] == 0
    _check(img_inf, full)


def test_block_tiles_follow_a_new_grid_of_the_same_size(cuda_device):
    """One processor, two grids with the same pixel count but different shapes (100 x 40
    and 40 x 100) under a finite band: the block tiling is re-planned for the second grid
    (a different number of tiles), and both images match the oracle."""
    import _sarlabtdc

    sc = scenes.small_scene(seed=94, n_pri=300, n_samples=32, nx=40, ny=100, rail_len=0.3, device="cuda")
    api = _moving_api(sc, speed=0.08)
    args = (0.0, 14.0, False, True, True)
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                 api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
    for nx, ny in ((40, 100), (100, 40)):
        grid = np.ascontiguousarray(scenes.ground_grid(nx, ny, 2e-3, y0=0.12).astype(np.float32))
        p.setFocusGrid(grid)
        p.start(*args)
        img = p.getFocusedImage()
        assert img.shape == (ny, nx)
        assert p.lastStats()["tile_cols"] == 16
        ref = _oracle(api, grid, args).reshape(img.shape)
        _check(img, ref, l2=2e-4, phase=None)


def test_unit_spans_skip_only_chirps_out_of_band_for_the_whole_tile(cuda_device):
    """Under a finite band each work unit visits only the chirps that some pixel of its tile can
    see in band (span_permille < 1000). The skipped chirps are out of band for every pixel, so
    the image is bit for bit the one without spans (chirp offsets of zero turn them off) and
    matches the oracle. A grid of the same shape moved along the rail gets spans of its own."""
    import torch

    import _sarlabtdc

    sc = scenes.small_scene(seed=95, n_pri=600, n_samples=128, nx=64, ny=48, rail_len=0.6, device="cuda")
    api = _moving_api(sc, speed=0.08)
    args = (0.0, 14.0, False, True, True)
    grid = sc.grid.astype(np.float32)

    def focus(offsets):
        p = _sarlabtdc.TdcProcessor(0)
        p.setRawData(*api.values())
        p.setFocusGrid(grid)
        p.prepare(*args)
        p.uploadGrid()
        if offsets:
            p.setChirpOffsetsDevice(torch.zeros((sc.n_pri, 3), dtype=torch.float64, device="cuda"))
        img = torch.empty(p.numPixels(), dtype=torch.complex64, device="cuda")
        p.focusDevice(img)
        p.check()
        return img.cpu().numpy(), p.lastStats()

    img, st = focus(False)
    img0, st0 = focus(True)
    assert st["tile_cols"] == 16 and st["span_permille"] < 700, st["span_permille"]
    assert st0["span_permille"] == 1000
    np.testing.assert_array_equal(img, img0)
    ref = _oracle(api, grid, args)
    _check(img, ref, l2=2e-4, phase=None)
    # the same processor, a grid of the same shape 0.1 m further along the rail
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setFocusGrid(grid)
    p.start(*args)
    moved = grid.copy()
    moved[..., 0] += 0.1
    p.setFocusGrid(moved)
    p.start(*args)
    assert p.lastStats()["span_permille"] < 1000
    _check(p.getFocusedImage(), _oracle(api, moved, args).reshape(moved.shape[:2]), l2=2e-4, phase=None)
