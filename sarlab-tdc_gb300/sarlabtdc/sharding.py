"""Pixel sharding of one focus across GPUs: one process per GPU (no reference counterpart;
the reference binds a single GPU, tdc-lib/src/tdcprocessor.cpp:39-55).

A focused pixel depends on the whole acquisition and on nothing else of the grid, so the
grid's rows are split into contiguous blocks, one per rank. Every rank holds the whole
acquisition (raw data, trajectory), focuses its own block on its own GPU with no data
moving between ranks, and the blocks are gathered once at the end. The work is sharded
with no collective on the data path: the gather moves only the finished image (8 bytes a
pixel).

Each rank plans its chirp groups for the whole grid's pixel count
(``TdcProcessor.setPlanPixels``), and every block starts on a multiple of 32 pixels (the
engine's anchored ranges share an anchor among up to 32 consecutive pixels of a grid). A
pixel's arithmetic then depends only on the chirp groups and its own group of 32 pixels, so
on GPUs of one kind the gathered image equals a single-GPU focus of the whole grid bit for
bit.
"""
from __future__ import annotations

import math

import numpy as np


def row_align(n_cols: int) -> int:
    """Rows per block step for a grid of n_cols columns: the fewest rows that hold a multiple
    of 32 pixels (1 when n_cols is a multiple of 32)."""
    return 32 // math.gcd(max(int(n_cols), 1), 32)


def row_blocks(n_rows: int, world_size: int, align: int = 1) -> list[tuple[int, int]]:
    """Contiguous [r0, r1) row blocks of a grid with n_rows rows, one per rank, each starting on
    a multiple of ``align`` rows: steps of ``align`` rows are shared out, the first
    (steps % world_size) blocks taking one step more, and the last non-empty block ends at
    n_rows (with fewer steps than ranks the last blocks are empty)."""
    if world_size < 1:
        raise ValueError("world_size must be at least 1")
    if n_rows < 0:
        raise ValueError("n_rows must not be negative")
    if align < 1:
        raise ValueError("align must be at least 1")
    steps = -(-n_rows // align)
    base, extra = divmod(steps, world_size)
    out, s0 = [], 0
    for k in range(world_size):
        s1 = s0 + base + (1 if k < extra else 0)
        out.append((min(s0 * align, n_rows), min(s1 * align, n_rows)))
        s0 = s1
    return out


def rank_rows(n_rows: int, world_size: int, rank: int, align: int = 1) -> tuple[int, int]:
    """The [r0, r1) row block of one rank."""
    if not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside 0..{world_size - 1}")
    return row_blocks(n_rows, world_size, align)[rank]


def gather_rows(local: np.ndarray, n_rows: int, n_cols: int, group=None) -> np.ndarray:
    """Assemble the [n_rows, n_cols] complex64 image from every rank's row block ``local``
    ([r1 - r0, n_cols]) with one all-gather of the default (or given) torch.distributed
    process group. Blocks are padded to the longest block for the collective. NCCL groups
    gather through the current CUDA device, others through host memory."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    blocks = row_blocks(n_rows, world, row_align(n_cols))
    rmax = max(r1 - r0 for r0, r1 in blocks)
    local = np.ascontiguousarray(local, dtype=np.complex64).reshape(-1, n_cols)
    rank = dist.get_rank(group)
    r0, r1 = blocks[rank]
    if local.shape[0] != r1 - r0:
        raise ValueError(f"rank {rank} holds {local.shape[0]} rows, its block is {r1 - r0}")
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" \
        else torch.device("cpu")
    buf = torch.zeros((rmax, n_cols, 2), dtype=torch.float32, device=dev)
    if local.size:
        buf[: r1 - r0] = torch.from_numpy(local.view(np.float32).reshape(-1, n_cols, 2)).to(dev)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = np.empty((n_rows, n_cols), dtype=np.complex64)
    for (b0, b1), part in zip(blocks, parts):
        if b1 > b0:
            out[b0:b1] = part[: b1 - b0].cpu().numpy().view(np.complex64).reshape(b1 - b0, n_cols)
    return out


class ShardedProcessor:
    """The reference's TdcProcessor interface over a row block of the focus grid, one per
    rank. ``setRawData`` takes the whole acquisition on every rank; ``setFocusGrid`` the whole
    grid (each rank keeps its block); ``start`` focuses the block; ``getFocusedImage``
    gathers the whole image on every rank (a collective: all ranks call it).

    ``processor`` is the per-rank engine (default: ``_sarlabtdc.TdcProcessor(gpuNum)``)."""

    def __init__(self, gpuNum: int, rank: int, world_size: int, group=None, processor=None):
        if processor is None:
            import _sarlabtdc

            processor = _sarlabtdc.TdcProcessor(gpuNum)
        self.proc = processor
        self.rank = int(rank)
        self.world_size = int(world_size)
        self.group = group
        self.rows = (0, 0)
        self.shape = (0, 0)

    def setRawData(self, *args):
        self.proc.setRawData(*args)

    def setChirpPositionsF64(self, position):
        self.proc.setChirpPositionsF64(position)

    def _set_grid(self, grid, setter):
        g = np.asarray(grid)
        if g.ndim != 3 or g.shape[2] != 3:
            raise RuntimeError("focusGrid shape is incorrect")
        n_rows, n_cols = g.shape[:2]
        r0, r1 = rank_rows(n_rows, self.world_size, self.rank, row_align(n_cols))
        self.rows = (r0, r1)
        self.shape = (n_rows, n_cols)
        setter(np.ascontiguousarray(g[r0:r1]))
        self.proc.setPlanPixels(n_rows * n_cols)

    def setFocusGrid(self, focusGrid):
        self._set_grid(focusGrid, self.proc.setFocusGrid)

    def setFocusGridF64(self, focusGrid):
        self._set_grid(focusGrid, self.proc.setFocusGridF64)

    def start(self, dopplerWinCenter, dopplerBandwidth, dopCentroidWin, applyRangeWin, dopplerWinTaper=True):
        self.proc.start(dopplerWinCenter, dopplerBandwidth, dopCentroidWin, applyRangeWin, dopplerWinTaper)

    def getLocalImage(self) -> np.ndarray:
        """This rank's row block [r1 - r0, n_cols] of the image."""
        r0, r1 = self.rows
        return np.asarray(self.proc.getFocusedImage()).reshape(r1 - r0, self.shape[1])

    def getFocusedImage(self) -> np.ndarray:
        return gather_rows(self.getLocalImage(), self.shape[0], self.shape[1], self.group)
