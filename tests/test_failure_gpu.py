"""Failure detection on the GPU without a fault: the kernels' bounded mbarrier wait gives
up on a barrier phase nothing completes, reports the timeout through the status word, and
the device stays usable (the next focus runs and matches the oracle)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from sarlabtdc import scenes
from tdc_testutil import problem_from_api, rel_l2, run_engine

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_device_stays_usable(cuda_device):
    import _tdc_capi

    L = _tdc_capi.lib()
    flag, ms = C.c_int(-1), C.c_double(0.0)
    _tdc_capi.check(L.tdc_selftest_wait_timeout(0, 50000, C.byref(flag), C.byref(ms)))
    assert flag.value == 1
    assert 45.0 <= ms.value < 1000.0, ms.value
    sc = scenes.small_scene(seed=41, n_pri=96, n_samples=40, nx=9, ny=7, device="cuda")
    api = sc.api_arrays()
    args = (0.0, float("inf"), False, True, True)
    img, stats, _ = run_engine(api, sc.grid, args)
    ref = oracle.focus(problem_from_api(api, sc.grid), oracle.Opts(applyRangeWin=True,
                                                                    dopplerBandwidth=float("inf")))
    assert rel_l2(img.ravel(), ref) <= 1e-4
