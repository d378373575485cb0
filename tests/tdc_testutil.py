"""Shared helpers of the test suite: run the engine and the oracle on one scene
and compare them with the accuracy metrics the engine is specified by."""
from __future__ import annotations

import numpy as np

import oracle


def rel_l2(a, b) -> float:
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def max_phase_err(a, b, floor_db=-40.0) -> float:
    """Largest |arg(a conj(b))| over pixels of b within floor_db of b's peak."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    m = np.abs(b)
    if m.max() == 0:
        return 0.0
    sel = m >= m.max() * 10 ** (floor_db / 20.0)
    return float(np.max(np.abs(np.angle(a[sel] * np.conj(b[sel])))))


def peak_err(a, b) -> float:
    ma, mb = np.abs(np.asarray(a)).max(), np.abs(np.asarray(b)).max()
    return float(abs(ma - mb) / (mb if mb > 0 else 1.0))


def problem_from_api(api: dict, grid, pos64=None, grid64=False) -> oracle.Problem:
    """Oracle problem with exactly the values the engine receives through setRawData."""
    pos = pos64 if pos64 is not None else api["position"]
    g = np.asarray(grid, np.float64 if grid64 else np.float32)
    return oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=pos,
                          velocity=api["velocity"], attitude=api["attitude"], modRate=api["modRate"],
                          startFreq=api["startFreq"], grid=g, bodyBoresight=tuple(api["bodyBoresight"]))


def run_engine(api: dict, grid, start_args, pos64=None, grid64=None, precision="fp32", skip_test=True, motion=True):
    import _sarlabtdc

    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                 api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
    if pos64 is not None:
        p.setChirpPositionsF64(pos64)
    if grid64 is not None:
        p.setFocusGridF64(grid64)
    else:
        p.setFocusGrid(grid)
    p.setPrecision(precision)
    p.setSkipTest(skip_test)
    p.setMotionPath(motion)
    p.start(*start_args)
    return p.getFocusedImage(), p.lastStats(), p
