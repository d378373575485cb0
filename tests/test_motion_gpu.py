"""GPU parity of the smooth-motion path (per-sample positions that move smoothly within
each chirp) against the FP64 oracle, which evaluates the range of every sample from its
own position as the reference does (tdc-lib/src/tdckernels.cu:202-216), and its routing:
what a quadratic in the sample index does not describe within FP32 rounding goes to the
FP32 general kernel.

Tolerances: relative L2 <= 1e-4 and max phase error <= 1e-3 rad over pixels within 40 dB
of the peak.
"""
import numpy as np
import pytest

import oracle
from sarlabtdc import scenes
from tdc_testutil import max_phase_err, problem_from_api, rel_l2, run_engine

pytestmark = pytest.mark.gpu

L2_TOL = 1e-4
PHASE_TOL = 1e-3
INF = float("inf")
START = (0.0, INF, False, True, True)


def _moving(sc, drift=0.3e-3, accel=0.0, seed=5):
    """Positions P_c + (s/S) delta_c + (s/S)^2 a_c: the antenna moving (and accelerating)
    during each chirp, stored as the API's FP32 per-sample positions."""
    rng = np.random.default_rng(seed)
    api = sc.api_arrays()
    C, S = sc.n_pri, sc.n_samples
    u = (np.arange(S) / S)[None, :, None]
    pos = api["position"].astype(np.float64) + u * rng.normal(0.0, drift, (C, 1, 3))
    if accel:
        pos = pos + u * u * rng.normal(0.0, accel, (C, 1, 3))
    api["position"] = pos.astype(np.float32)
    return api


def _oracle(api, grid, args=START):
    c, b, cw, rw, tp = args
    return oracle.focus(problem_from_api(api, grid), oracle.Opts(dopplerWinCenter=c, dopplerBandwidth=b,
                                                                 dopCentroidWin=cw, applyRangeWin=rw,
                                                                 dopplerWinTaper=tp))


def _check(img, ref):
    e = rel_l2(img, ref)
    assert e <= L2_TOL, f"relative L2 {e:.3e}"
    p = max_phase_err(img, ref)
    assert p <= PHASE_TOL, f"max phase error {p:.3e} rad"
    return e


@pytest.mark.parametrize("n_samples,drift", [(64, 0.3e-3), (256, 0.3e-3), (1024, 0.3e-3), (1024, 0.7e-3),
                                             (1500, 0.5e-3), (4000, 0.2e-3)])
def test_smooth_motion_against_the_oracle(cuda_device, n_samples, drift):
    """Linear drift within each chirp (0.2-0.7 mm), rows of 64-4000 samples, ragged tile."""
    sc = scenes.small_scene(seed=200 + n_samples, n_pri=192, n_samples=n_samples, nx=21, ny=19, jitter=0.2e-3,
                            device="cuda")
    api = _moving(sc, drift=drift)
    img, stats, _ = run_engine(api, sc.grid, START)
    assert stats["path_name"] == "fp32_motion"
    seg = stats["motion_segment"]
    assert seg >= 8 and seg & (seg - 1) == 0
    ref = _oracle(api, sc.grid).reshape(img.shape)
    _check(img, ref)
    # the FP32 general kernel on the same inputs agrees with both
    gen, gstats, _ = run_engine(api, sc.grid, START, motion=False)
    assert gstats["path_name"] == "general"
    _check(gen, ref)


def test_accelerating_antenna_against_the_oracle(cuda_device):
    """A quadratic in the sample index (acceleration within the chirp) is fitted exactly."""
    sc = scenes.small_scene(seed=210, n_pri=160, n_samples=512, nx=19, ny=17, device="cuda")
    api = _moving(sc, drift=0.3e-3, accel=0.4e-3)
    img, stats, _ = run_engine(api, sc.grid, START)
    assert stats["path_name"] == "fp32_motion"
    _check(img, _oracle(api, sc.grid).reshape(img.shape))


def test_motion_beyond_a_quadratic_takes_the_general_kernel(cuda_device):
    """A vibration (a sine over the chirp, 20 um) is not a quadratic: the FP32 general
    kernel runs, with the oracle's result."""
    sc = scenes.small_scene(seed=211, n_pri=128, n_samples=256, nx=16, ny=12, device="cuda")
    api = _moving(sc, drift=0.2e-3)
    S = sc.n_samples
    pos = api["position"].astype(np.float64)
    pos[..., 2] += 20e-6 * np.sin(2 * np.pi * 3 * np.arange(S) / S)[None, :]
    api["position"] = pos.astype(np.float32)
    img, stats, _ = run_engine(api, sc.grid, START)
    assert stats["path_name"] == "general"
    _check(img, _oracle(api, sc.grid).reshape(img.shape))


def test_finite_band_on_a_still_antenna(cuda_device):
    """Zero velocity: the Doppler frequency is 0 for every sample, so a finite band is one
    window per chirp (the zero-window-skipping instance runs): a band around 0 gives the
    tapered weight the oracle gives, a band away from 0 an all-zero image."""
    sc = scenes.small_scene(seed=212, n_pri=200, n_samples=128, nx=17, ny=13, device="cuda")
    api = _moving(sc, drift=0.3e-3)
    args = (1.0, 6.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    assert stats["path_name"] == "fp32_motion"
    _check(img, _oracle(api, sc.grid, args).reshape(img.shape))
    args_out = (40.0, 6.0, False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args_out)
    assert stats["path_name"] == "fp32_motion"
    assert not np.any(img)
    assert not np.any(_oracle(api, sc.grid, args_out))


def test_long_rows_beyond_whole_row_stages_take_the_general_kernel(cuda_device):
    """Rows too long for whole-row stages (12,000 samples) go to the general kernel, which
    stages them in segments; 8,000-sample rows stay on the smooth-motion kernel."""
    for n_samples, path in ((8000, "fp32_motion"), (12000, "general")):
        sc = scenes.small_scene(seed=213, n_pri=24, n_samples=n_samples, nx=9, ny=7, rail_len=0.1, device="cuda")
        api = _moving(sc, drift=0.1e-3)
        img, stats, _ = run_engine(api, sc.grid, START)
        assert stats["path_name"] == path
        _check(img, _oracle(api, sc.grid).reshape(img.shape))


def test_smooth_motion_repeatable_and_linear(cuda_device):
    sc = scenes.small_scene(seed=214, n_pri=256, n_samples=96, nx=24, ny=20, device="cuda")
    api = _moving(sc, drift=0.3e-3)
    a, _, _ = run_engine(api, sc.grid, START)
    b, _, _ = run_engine(api, sc.grid, START)
    np.testing.assert_array_equal(a, b)
    api2 = dict(api)
    api2["rawData"] = (api["rawData"] * np.float32(2.0)).astype(np.complex64)
    c, _, _ = run_engine(api2, sc.grid, START)
    np.testing.assert_array_equal(c, 2 * a)
