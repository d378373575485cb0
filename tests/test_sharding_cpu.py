"""CPU tests of pixel sharding across ranks (sarlabtdc.sharding): the row partition, and two
gloo ranks that each focus their row block -- the FP64 oracle standing in for the GPU
engine behind the processor interface -- and gather the image, which must equal the
single-rank image bit for bit (each pixel's value does not depend on the rest of the grid).
"""
import os
import socket

import numpy as np
import pytest

import oracle
from sarlabtdc import scenes, sharding
from tdc_testutil import problem_from_api

INF = float("inf")
START = (0.0, INF, False, True, True)


def test_row_blocks_cover_the_grid_in_order():
    for n_rows in (0, 1, 2, 7, 13, 1024):
        for world in (1, 2, 3, 8):
            blocks = sharding.row_blocks(n_rows, world)
            assert len(blocks) == world
            assert blocks[0][0] == 0 and blocks[-1][1] == n_rows
            sizes = [r1 - r0 for r0, r1 in blocks]
            assert all(s >= 0 for s in sizes) and max(sizes) - min(sizes) <= 1
            assert all(blocks[k][1] == blocks[k + 1][0] for k in range(world - 1))
            for rank in range(world):
                assert sharding.rank_rows(n_rows, world, rank) == blocks[rank]
    with pytest.raises(ValueError):
        sharding.row_blocks(4, 0)
    with pytest.raises(ValueError):
        sharding.rank_rows(4, 2, 2)


def test_row_blocks_start_on_multiples_of_32_pixels():
    """Blocks start on whole steps of row_align(n_cols) rows, so every block's first pixel is a
    multiple of 32 (the engine's anchor groups are the same in a block as in the whole grid)."""
    assert [sharding.row_align(c) for c in (1024, 96, 16, 9, 48, 1)] == [1, 1, 2, 32, 2, 32]
    for n_rows in (0, 1, 5, 13, 100, 1023):
        for n_cols in (9, 16, 48, 100, 256):
            a = sharding.row_align(n_cols)
            for world in (1, 2, 3, 5):
                blocks = sharding.row_blocks(n_rows, world, a)
                assert blocks[0][0] == 0 and max(r1 for _, r1 in blocks) == n_rows
                assert all(blocks[k][1] == blocks[k + 1][0] for k in range(world - 1))
                for r0, r1 in blocks:
                    assert r0 <= r1 and (r0 * n_cols) % 32 == 0 or r0 == n_rows
                sizes = [r1 - r0 for r0, r1 in blocks]
                assert max(sizes) - min(sizes) <= 2 * a - 1  # (the last block ends at n_rows)
    assert sharding.row_blocks(13, 2, 2) == [(0, 8), (8, 13)]
    with pytest.raises(ValueError):
        sharding.row_blocks(4, 2, 0)


class OracleProcessor:
    """The processor interface with the FP64 oracle computing the focus (a CPU stand-in for
    the GPU engine, test infrastructure only)."""

    def setRawData(self, rawData, priTimes, sampleTimes, position, velocity, attitude, modRate, startFreq,
                   bodyBoresight):
        self.api = dict(rawData=rawData, priTimes=priTimes, sampleTimes=sampleTimes, position=position,
                        velocity=velocity, attitude=attitude, modRate=modRate, startFreq=startFreq,
                        bodyBoresight=bodyBoresight)

    def setFocusGrid(self, grid):
        self.grid = np.asarray(grid, np.float32)

    def setPlanPixels(self, n_pix):
        self.plan_pixels = n_pix

    def start(self, c, b, cw, rw, taper=True):
        o = oracle.Opts(dopplerWinCenter=c, dopplerBandwidth=b, dopCentroidWin=cw, applyRangeWin=rw,
                        dopplerWinTaper=taper)
        if self.grid.size:
            img = oracle.focus(problem_from_api(self.api, self.grid), o, threads=1)
        else:
            img = np.zeros(0, np.complex128)
        self.img = img.astype(np.complex64).reshape(self.grid.shape[:2])

    def getFocusedImage(self):
        return self.img


def _scene():
    sc = scenes.small_scene(seed=17, n_pri=96, n_samples=48, nx=16, ny=13, jitter=0.2e-3)
    return sc, sc.api_arrays()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc, api = _scene()
        sp = sharding.ShardedProcessor(0, rank, world, processor=OracleProcessor())
        sp.setRawData(*api.values())
        sp.setFocusGrid(sc.grid.astype(np.float32))
        assert sp.proc.plan_pixels == sc.grid.shape[0] * sc.grid.shape[1]
        sp.start(*START)
        local = sp.getLocalImage()
        img = sp.getFocusedImage()
        np.save(os.path.join(out_dir, f"local{rank}.npy"), local)
        np.save(os.path.join(out_dir, f"image{rank}.npy"), img)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_gather_the_single_rank_image(tmp_path, world):
    """world_size 2 (13 rows of 16 pixels: blocks of 8 and 5 rows) and 3 over gloo, one process
    per rank."""
    import torch.multiprocessing as mp

    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    sc, api = _scene()
    single = OracleProcessor()
    single.setRawData(*api.values())
    single.setFocusGrid(sc.grid)
    single.start(*START)
    full = single.getFocusedImage()
    blocks = sharding.row_blocks(full.shape[0], world, sharding.row_align(full.shape[1]))
    for rank in range(world):
        np.testing.assert_array_equal(np.load(tmp_path / f"image{rank}.npy"), full)
        r0, r1 = blocks[rank]
        np.testing.assert_array_equal(np.load(tmp_path / f"local{rank}.npy"), full[r0:r1])
