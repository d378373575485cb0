"""GPU parity of the FP32-bulk kernel's anchored ranges: groups of 32 consecutive pixels
share an anchor pixel whose range and phase terms are formed in double-float once per chirp,
and each pixel adds its FP32 range difference from the anchor. Checked against the FP64
oracle and against the same focus with every (pixel, chirp) range in double-float
(setAnchoredRanges(False)): anchoring may cost at most a factor 2 of the engine's own error."""
import numpy as np
import pytest

import oracle
from sarlabtdc import scenes
from tdc_testutil import max_phase_err, problem_from_api, rel_l2

pytestmark = pytest.mark.gpu

INF = float("inf")
ARGS = (0.0, INF, False, False, True)


def _oracle(api, grid, pos64=None, grid64=False):
    o = oracle.Opts(dopplerWinCenter=0.0, dopplerBandwidth=INF, dopCentroidWin=False, applyRangeWin=False,
                    dopplerWinTaper=True)
    return oracle.focus(problem_from_api(api, grid, pos64=pos64, grid64=grid64), o)


def _focus(api, grid, anchored, pos64=None, grid64=False):
    import _sarlabtdc

    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    if pos64 is not None:
        p.setChirpPositionsF64(pos64)
    if grid64:
        p.setFocusGridF64(grid)
    else:
        p.setFocusGrid(grid)
    p.setAnchoredRanges(anchored)
    p.start(*ARGS)
    return p.getFocusedImage(), p.lastStats()


def _compare(api, grid, group, pos64=None, grid64=False):
    img, st = _focus(api, grid, True, pos64, grid64)
    assert st["path_name"] == "fp32_bulk" and st["anchor_pixels"] == group
    ref = _oracle(api, grid, pos64, grid64).reshape(img.shape)
    if group == 0:
        assert rel_l2(img, ref) <= 1e-4
        return
    plain, st0 = _focus(api, grid, False, pos64, grid64)
    assert st0["anchor_pixels"] == 0
    e_anchor, e_plain = rel_l2(img, ref), rel_l2(plain, ref)
    assert e_anchor <= max(2.0 * e_plain, 5e-6), (e_anchor, e_plain)
    assert max_phase_err(img, ref) <= 1e-3
    return e_anchor, e_plain


@pytest.mark.parametrize("n_samples,group", [(128, 32), (256, 32), (512, 32), (640, 32), (1024, 0), (2048, 0)])
def test_anchor_groups_against_oracle(cuda_device, n_samples, group):
    """Rows staged 15, 7, 4 and 3 chirps a stage (one or two passes of anchor records), and none
    at 1 or 2 chirps a stage, where the double-float instance is faster; on a 19 x 57 grid at
    1 mm: rows of 19 pixels (1.9 cm), so groups wrap rows and stay within the anchor bounds, and
    1,083 pixels end in a partial tile and a partial group."""
    sc = scenes.small_scene(seed=40 + n_samples, n_pri=96, n_samples=n_samples, nx=19, ny=57, jitter=0.3e-3,
                            spacing=1e-3, device="cuda")
    _compare(sc.api_arrays(), sc.grid.astype(np.float32), group)


def test_anchor_fp64_grid_and_positions(cuda_device):
    """FP64 grid and chirp positions (double-float pixel coordinates and antenna positions)."""
    sc = scenes.small_scene(seed=77, n_pri=128, n_samples=256, nx=32, ny=30, jitter=0.5e-3, device="cuda")
    _compare(sc.api_arrays(), sc.grid, 32, pos64=sc.positions, grid64=True)


def test_antenna_on_a_pixel(cuda_device):
    """One chirp's antenna exactly on a pixel: its range is zero there and its Doppler window NaN,
    so that chirp contributes nothing to that pixel (the reference's NaN -> 0 window) and the
    other pixels of the anchor group stay finite."""
    sc = scenes.small_scene(seed=78, n_pri=64, n_samples=256, nx=32, ny=8, device="cuda")
    api = sc.api_arrays()
    grid = sc.grid.astype(np.float32)
    api["position"] = np.array(api["position"])
    api["position"][10, :, :] = grid[3, 5]
    img, _ = _focus(api, grid, True)
    assert np.all(np.isfinite(img))
    _compare(api, grid, 32)


def test_far_apart_pixels_take_double_float_ranges(cuda_device):
    """Pixels 6 mm apart put 32-pixel groups beyond the 5 cm anchor bound, and so do rows of
    45 pixels at 2 mm (groups that wrap a row hold pixels from both of its ends): every range
    is then formed in double-float."""
    sc = scenes.small_scene(seed=82, n_pri=64, n_samples=256, nx=45, ny=6, device="cuda")
    _, st = _focus(sc.api_arrays(), sc.grid.astype(np.float32), True)
    assert st["anchor_pixels"] == 0
    sc = scenes.small_scene(seed=79, n_pri=64, n_samples=256, nx=40, ny=6, spacing=6e-3, device="cuda")
    img, st = _focus(sc.api_arrays(), sc.grid.astype(np.float32), True)
    assert st["anchor_pixels"] == 0
    ref = _oracle(sc.api_arrays(), sc.grid.astype(np.float32)).reshape(img.shape)
    assert rel_l2(img, ref) <= 1e-4


def test_short_rows_and_finite_band_take_double_float_ranges(cuda_device):
    """More than 16 chirps a stage (rows of 64 samples) and a finite Doppler band keep the
    per-pixel double-float ranges."""
    import _sarlabtdc

    sc = scenes.small_scene(seed=80, n_pri=64, n_samples=64, nx=24, ny=8, device="cuda")
    _, st = _focus(sc.api_arrays(), sc.grid.astype(np.float32), True)
    assert st["anchor_pixels"] == 0 and st["stage_chirps"] > 16
    sc = scenes.small_scene(seed=81, n_pri=64, n_samples=256, nx=24, ny=8, device="cuda")
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*sc.api_arrays().values())
    p.setFocusGrid(sc.grid.astype(np.float32))
    p.start(0.0, 40.0, False, False, True)
    assert p.lastStats()["anchor_pixels"] == 0
