"""Pixel sharding on the GPU: the row blocks of a grid, focused one after another on this
GPU as the ranks of a sharded focus would focus them (blocks are independent: no rank waits
for another), assemble into the whole grid's image bit for bit when each block plans its
chirp groups for the whole grid (ShardedProcessor does), and agree with it to FP32 rounding
when each plans for itself."""
import numpy as np
import pytest

from sarlabtdc import scenes, sharding
from tdc_testutil import rel_l2

pytestmark = pytest.mark.gpu

START = (0.0, float("inf"), False, True, True)


class _NoGroupSharded(sharding.ShardedProcessor):
    """A rank's processor without a process group: the blocks are assembled by the test."""


def _focus_blocks(sc, api, world, pin):
    import _sarlabtdc

    out = np.empty(sc.grid.shape[:2], np.complex64)
    for rank in range(world):
        sp = _NoGroupSharded(0, rank, world)
        sp.setRawData(*api.values())
        sp.setFocusGrid(sc.grid.astype(np.float32))
        if not pin:
            sp.proc.setPlanPixels(0)
        sp.start(*START)
        r0, r1 = sp.rows
        out[r0:r1] = sp.getLocalImage()
        assert isinstance(sp.proc, _sarlabtdc.TdcProcessor)
    return out


@pytest.mark.parametrize("world", [2, 3, 5])
def test_blocks_assemble_the_whole_grid_bit_for_bit(cuda_device, world):
    import _sarlabtdc

    sc = scenes.small_scene(seed=301, n_pri=1024, n_samples=128, nx=128, ny=257, jitter=0.2e-3, device="cuda")
    api = sc.api_arrays()
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setFocusGrid(sc.grid.astype(np.float32))
    p.start(*START)
    whole = p.getFocusedImage()
    np.testing.assert_array_equal(_focus_blocks(sc, api, world, pin=True), whole)
    # planned per block, the chirp groups (each pixel's summation order) may differ: FP32 rounding
    assert rel_l2(_focus_blocks(sc, api, world, pin=False), whole) < 1e-6


@pytest.mark.parametrize("world", [2, 3])
def test_anchored_blocks_assemble_the_whole_grid_bit_for_bit(cuda_device, world):
    """With anchored ranges (32 consecutive pixels share an anchor) on a grid of 40 columns:
    the blocks start on multiples of 32 pixels (4 rows), so every pixel keeps its anchor and
    the assembled image equals the whole grid's bit for bit."""
    import _sarlabtdc

    sc = scenes.small_scene(seed=302, n_pri=512, n_samples=256, nx=40, ny=57, jitter=0.2e-3, spacing=1e-3,
                            device="cuda")
    api = sc.api_arrays()
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setFocusGrid(sc.grid.astype(np.float32))
    p.start(*START)
    assert p.lastStats()["anchor_pixels"] == 32
    whole = p.getFocusedImage()
    assert sharding.row_align(40) == 4
    np.testing.assert_array_equal(_focus_blocks(sc, api, world, pin=True), whole)


def test_finite_band_blocks_assemble_the_whole_grid_bit_for_bit(cuda_device):
    """Under a finite Doppler band with the antenna moving along the rail, each row block plans
    its own block tiles and unit spans (the chirps its tiles can see in band); neither changes
    a pixel's sums, so the blocks assemble into the whole grid's image bit for bit."""
    import _sarlabtdc

    sc = scenes.small_scene(seed=303, n_pri=600, n_samples=128, nx=64, ny=96, rail_len=0.6, device="cuda")
    api = sc.api_arrays()
    vel = np.zeros((sc.n_pri, sc.n_samples, 3), np.float32)
    vel[..., 0] = 0.08
    api["velocity"] = vel
    args = (0.0, 14.0, False, True, True)
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setFocusGrid(sc.grid.astype(np.float32))
    p.start(*args)
    st = p.lastStats()
    assert st["tile_cols"] == 16 and st["span_permille"] < 1000
    whole = p.getFocusedImage()
    out = np.empty_like(whole)
    for rank in range(3):
        sp = _NoGroupSharded(0, rank, 3)
        sp.setRawData(*api.values())
        sp.setFocusGrid(sc.grid.astype(np.float32))
        sp.start(*args)
        r0, r1 = sp.rows
        out[r0:r1] = sp.getLocalImage()
    np.testing.assert_array_equal(out, whole)
