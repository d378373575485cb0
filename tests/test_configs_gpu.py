"""GPU parity at the benchmark configurations' own sizes.

Each test builds one benchmark scene at full size (the seeded generators in
sarlabtdc.scenes), focuses it through the reference-shaped module
(_sarlabtdc.TdcProcessor, or the request loop for the serving mix), and checks
a seeded pixel subset -- every target's nearest pixel plus at least 2,048
random pixels -- against the FP64 oracle on the same inputs. The call follows
tdc-lib/src/tdcprocessor.cpp:59-167 as the benchmarks use it: the Hann window is
already applied to the raw data, applyRangeWin = False, infinite Doppler band.

These catch what only shows at configuration scale: millions of pixels in
thousands of tiles, chirp groups of 16,384 chirps, 256-sample rows several
chirps to a stage, 2048^2 grids with 8192 chirps in a mixed launch.

Tolerances: relative L2 <= 1e-4 and max phase error <= 1e-3 rad over pixels of
the subset within 40 dB of its peak.
"""
import numpy as np
import pytest

import oracle
from sarlabtdc import scenes
from tdc_testutil import max_phase_err, peak_err, rel_l2

pytestmark = pytest.mark.gpu

L2_TOL = 1e-4
PHASE_TOL = 1e-3
INF = float("inf")
START = (0.0, INF, False, False, True)
N_RANDOM = 2048


def _subset(grid, targets, n_random, seed):
    """Flat indices of the pixel nearest each target plus n_random seeded random pixels."""
    from scipy.spatial import cKDTree

    flat = np.asarray(grid, np.float64).reshape(-1, 3)
    near = cKDTree(flat).query(np.asarray(targets, np.float64))[1]
    rnd = np.random.default_rng(seed).choice(flat.shape[0], size=min(n_random, flat.shape[0]), replace=False)
    return np.unique(np.concatenate([np.asarray(near, np.int64).ravel(), rnd.astype(np.int64)]))


def _check(got, ref):
    e_l2 = rel_l2(got, ref)
    e_ph = max_phase_err(got, ref)
    assert e_l2 <= L2_TOL, f"relative L2 {e_l2:.3e} > {L2_TOL:.0e}"
    assert e_ph <= PHASE_TOL, f"max phase error {e_ph:.3e} rad > {PHASE_TOL:.0e}"
    return e_l2, e_ph


def _processor(api, grid32=None, pos64=None, grid64=None):
    import _sarlabtdc

    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                 api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
    if pos64 is not None:
        p.setChirpPositionsF64(pos64)
    if grid64 is not None:
        p.setFocusGridF64(grid64)
    else:
        p.setFocusGrid(grid32)
    p.start(*START)
    return p


def _oracle_fp32_api(api, grid32, pixels):
    """Oracle on the FP32 API values: per-chirp positions (the broadcast rows are equal)."""
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=api["position"][:, 0, :],
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=grid32)
    return oracle.focus(prob, oracle.Opts(applyRangeWin=False, dopplerBandwidth=INF), pixels=pixels)


def test_config1_stripmap_full_grid(cuda_device):
    """256 x 256 ground grid at 2 mm, 1024 chirps x 512 samples on a 0.5 m rail, FP32 API
    inputs: every pixel against the oracle (34 Gcorr on the host cores)."""
    sc = scenes.stripmap(device="cuda")
    api = sc.api_arrays()
    grid32 = sc.grid.astype(np.float32)
    p = _processor(api, grid32=grid32)
    assert p.lastStats()["path_name"] == "fp32_bulk"
    img = p.getFocusedImage()
    assert img.shape == (256, 256)
    ref = _oracle_fp32_api(api, grid32, None).reshape(img.shape)
    _check(img, ref)
    assert peak_err(img, ref) <= 1e-4


def test_config2_precision_study_pixel_subset(cuda_device):
    """1024 x 1024 grid at 1 mm, 4096 chirps x 1024 samples over 2 m with 0.5 mm jitter, FP64
    positions and grid through the extensions; 50 targets + 2,048 random pixels."""
    sc = scenes.precision_study(device="cuda")
    api = sc.api_arrays()
    p = _processor(api, pos64=sc.positions, grid64=sc.grid)
    st = p.lastStats()
    assert st["path_name"] == "fp32_bulk"
    img = p.getFocusedImage().ravel()
    pix = _subset(sc.grid, sc.targets, N_RANDOM, seed=102)
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid)
    ref = oracle.focus(prob, oracle.Opts(applyRangeWin=False, dopplerBandwidth=INF), pixels=pix)
    _check(img[pix], ref)


def test_config3_volume_pixel_subset(cuda_device):
    """3-D near field: 128 x 128 planar aperture (16,384 chirps) x 256 samples, 256 x 256 x 64
    voxels flattened to a 16384 x 256 grid of points; 200 scatterers + 2,048 random voxels."""
    sc = scenes.volume_3d(device="cuda")
    api = sc.api_arrays()
    grid32 = sc.grid.astype(np.float32)
    p = _processor(api, grid32=grid32)
    assert p.lastStats()["path_name"] == "fp32_bulk"
    img = p.getFocusedImage()
    assert img.shape == (16384, 256)
    pix = _subset(sc.grid, sc.targets, N_RANDOM, seed=103)
    ref = _oracle_fp32_api(api, grid32, pix)
    _check(img.ravel()[pix], ref)


def test_config5_autofocus_scene_forward_pixel_subset(cuda_device):
    """The autofocus scene's forward focus on the nominal trajectory (512 x 512 at 1 mm,
    4096 chirps x 1024 samples, FP64 positions and grid): 30 targets + 2,048 random pixels.
    The data carry the random-walk trajectory error, so this is a defocused image; parity
    holds all the same."""
    sc = scenes.autofocus_scene(device="cuda")
    api = sc.api_arrays()
    p = _processor(api, pos64=sc.positions, grid64=sc.grid)
    img = p.getFocusedImage().ravel()
    pix = _subset(sc.grid, sc.targets, N_RANDOM, seed=105)
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid)
    ref = oracle.focus(prob, oracle.Opts(applyRangeWin=False, dopplerBandwidth=INF), pixels=pix)
    _check(img[pix], ref)


def _serving_job(side, n_pri, n_samples, n_targets, seed):
    """One request of the serving mix as the benchmark draws them: a rail at 0.25 mm spacing
    0.3 m above a side x side grid spanning 1 m from y = 0.3 m, FP32 inputs."""
    rng = np.random.default_rng(seed)
    radar = scenes.Radar(n_samples=n_samples)
    pos = scenes.rail(n_pri, n_pri * 0.25e-3, 0.3)
    grid = scenes.ground_grid(side, side, 1.0 / side, y0=0.3).astype(np.float32)
    lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
    tg = np.zeros((n_targets, 3))
    tg[:, 0] = rng.uniform(lo[0], hi[0], n_targets)
    tg[:, 1] = rng.uniform(lo[1], hi[1], n_targets)
    amps = np.exp(2j * np.pi * rng.uniform(0, 1, n_targets))
    raw = scenes.simulate_raw(pos, tg, amps, radar, "cuda").astype(np.complex64)
    return dict(raw=raw, st=radar.sample_times(), pos=pos.astype(np.float32), grid=grid, targets=tg,
                K=np.float32(radar.mod_rate), f0=np.float32(radar.f0))


def test_config4_serving_mix_extremes_against_oracle(cuda_device):
    """Four requests from the serving mix's range submitted at once to the request loop
    (they share launches): 2048^2 px x 8192 chirps x 1024 samples, 128^2 x 256 x 256, and two
    in between. Each image's subset is checked against the oracle."""
    from sarlabtdc.serving import FocusServer

    shapes = [(2048, 8192, 1024, 100, 41), (128, 256, 256, 1, 42), (512, 1024, 512, 30, 43),
              (1024, 2896, 256, 60, 44)]
    jobs = [_serving_job(*s) for s in shapes]
    with FocusServer(max_jobs=4) as srv:
        ids = [srv.submit(j["raw"], j["st"], j["pos"], j["grid"], j["K"], j["f0"], start=START) for j in jobs]
        results = [srv.wait(i) for i in ids]
    for (side, n_pri, n_samples, _, seed), j, (img, info) in zip(shapes, jobs, results):
        assert info["status"] == 0
        assert img.size == side * side
        pix = _subset(j["grid"], j["targets"], N_RANDOM, seed=seed)
        prob = oracle.Problem(raw=j["raw"], sampleTimes=j["st"], position=j["pos"], modRate=j["K"],
                              startFreq=j["f0"], grid=j["grid"])
        ref = oracle.focus(prob, oracle.Opts(applyRangeWin=False, dopplerBandwidth=INF), pixels=pix)
        _check(img[pix], ref)
