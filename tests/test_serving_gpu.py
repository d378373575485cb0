"""GPU tests of the request loop: results identical alone and in a mix,
memory-based admission, overlap of a job arriving while another runs, and
rejection of a job larger than the budget."""
import time

import numpy as np
import pytest

from sarlabtdc import scenes

pytestmark = pytest.mark.gpu

START = (0.0, float("inf"), False, False, True)


def _jobs():
    shapes = [  # (nx, ny, n_pri, n_samples, seed)
        (64, 48, 384, 256, 1), (100, 37, 160, 128, 2), (32, 32, 900, 64, 3),
        (128, 128, 256, 512, 4), (17, 5, 1024, 32, 5), (96, 80, 512, 96, 6),
    ]
    out = []
    for nx, ny, C, S, seed in shapes:
        sc = scenes.small_scene(seed=seed, n_pri=C, n_samples=S, nx=nx, ny=ny, jitter=0.2e-3, device="cuda")
        out.append(sc)
    return out


def _submit(srv, sc, f64=True):
    return srv.submit(sc.raw, sc.radar.sample_times(), sc.positions if f64 else sc.positions.astype(np.float32),
                      sc.grid if f64 else sc.grid.astype(np.float32), np.float32(sc.radar.mod_rate),
                      np.float32(sc.radar.f0), start=START)


def test_same_result_alone_and_in_mix_and_as_processor(cuda_device):
    import _sarlabtdc
    from sarlabtdc.serving import FocusServer

    jobs = _jobs()
    with FocusServer(max_jobs=4) as srv:
        alone = []
        for sc in jobs:
            img, info = srv.wait(_submit(srv, sc))
            assert info["status"] == 0
            alone.append(img)
        ids = [_submit(srv, sc) for sc in jobs]          # all at once: they share launches
        mixed = [srv.wait(i)[0] for i in ids]
        st = srv.stats()
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(a, m)
    assert st["jobs_done"] == 2 * len(jobs)
    # and the same as the processor (tdc_processor_focus_device path)
    for sc, a in zip(jobs, alone):
        p = _sarlabtdc.TdcProcessor(0)
        api = sc.api_arrays()
        p.setRawData(*api.values())
        p.setChirpPositionsF64(sc.positions)
        p.setFocusGridF64(sc.grid)
        p.start(*START)
        np.testing.assert_array_equal(p.getFocusedImage().ravel(), a)


def test_admission_under_a_tight_budget(cuda_device):
    from sarlabtdc.serving import FocusServer

    jobs = _jobs()
    budget = 96 << 20
    with FocusServer(memory_budget=budget, max_jobs=6) as srv:
        ids = [_submit(srv, sc) for sc in jobs]
        peak = 0
        while True:
            st = srv.stats()
            peak = max(peak, st["device_bytes_in_use"])
            if st["jobs_done"] + st["jobs_failed"] == len(jobs):
                break
            time.sleep(0.002)
        for i in ids:
            img, info = srv.wait(i)
            assert info["status"] == 0 and np.isfinite(img).all()
    assert peak <= budget


def test_job_arriving_during_a_long_job_overlaps_it(cuda_device):
    from sarlabtdc.serving import FocusServer

    long = scenes.small_scene(seed=9, n_pri=4096, n_samples=512, nx=1536, ny=1536, device="cuda")
    short = scenes.small_scene(seed=10, n_pri=256, n_samples=128, nx=32, ny=32, device="cuda")
    with FocusServer(max_jobs=4) as srv:
        lid = _submit(srv, long)
        time.sleep(0.05)
        sid = _submit(srv, short)
        _, si = srv.wait(sid)
        _, li = srv.wait(lid)
    assert si["first_launch_ms"] < li["done_ms"]      # started while the long job was on the GPU
    assert si["done_ms"] < li["done_ms"]              # and finished before it


def test_job_over_budget_fails_alone(cuda_device):
    from sarlabtdc.serving import FocusServer

    big = scenes.small_scene(seed=11, n_pri=512, n_samples=512, nx=256, ny=256, device="cuda")
    small = scenes.small_scene(seed=12, n_pri=128, n_samples=64, nx=16, ny=16, device="cuda")
    with FocusServer(memory_budget=8 << 20, max_jobs=2) as srv:
        bid = _submit(srv, big)
        sid = _submit(srv, small)
        with pytest.raises(MemoryError):
            srv.wait(bid)
        img, info = srv.wait(sid)
        assert info["status"] == 0


def _jittered_times(sc, seed):
    st = sc.radar.sample_times().astype(np.float64)
    st += np.random.default_rng(seed).uniform(-0.3, 0.3, st.shape) * (st[1] - st[0])
    return st.astype(np.float32)


def _processor_image(sc, sample_times=None):
    import _sarlabtdc

    p = _sarlabtdc.TdcProcessor(0)
    api = sc.api_arrays()
    if sample_times is not None:
        api["sampleTimes"] = sample_times
    p.setRawData(*api.values())
    p.setChirpPositionsF64(sc.positions)
    p.setFocusGridF64(sc.grid)
    p.start(*START)
    return p.getFocusedImage().ravel(), p.lastStats()


def test_general_and_long_row_jobs_are_batched_by_kind(cuda_device):
    """Jobs the FP32-bulk kernel cannot take whole (jittered sample times: the FP32 general
    kernel; rows too long for the stages: the segmented kernel) are batched with jobs of their
    own kind, beside the bulk launches, and each gives the processor's image bit for bit."""
    from sarlabtdc.serving import FocusServer

    bulk = _jobs()[:2]
    odd = [scenes.small_scene(seed=13 + k, n_pri=300, n_samples=96, nx=40, ny=30, jitter=0.2e-3, device="cuda")
           for k in range(2)]
    odd_t = [_jittered_times(sc, 4 + k) for k, sc in enumerate(odd)]
    long_row = scenes.small_scene(seed=15, n_pri=48, n_samples=9600, nx=24, ny=16, jitter=0.2e-3, device="cuda")
    with FocusServer(max_jobs=6) as srv:
        ids = [_submit(srv, sc) for sc in bulk]
        oids = [srv.submit(sc.raw, st, sc.positions, sc.grid, np.float32(sc.radar.mod_rate),
                           np.float32(sc.radar.f0), start=START) for sc, st in zip(odd, odd_t)]
        lid = _submit(srv, long_row)
        odd_out = [srv.wait(i) for i in oids]
        long_img, long_info = srv.wait(lid)
        for i in ids:
            assert srv.wait(i)[1]["status"] == 0
        stats = srv.stats()
    assert stats["unbatched"] == 0
    for sc, st, (img, info) in zip(odd, odd_t, odd_out):
        assert info["status"] == 0 and info["path"] == 2
        ref, pst = _processor_image(sc, st)
        assert pst["path_name"] == "general"
        np.testing.assert_array_equal(ref, img)
    assert long_info["status"] == 0 and long_info["path"] == 0
    ref, pst = _processor_image(long_row)
    assert pst["stage_chirps"] == 1 and pst["stage_samples"] < 9600
    np.testing.assert_array_equal(ref, long_img)


def test_finite_band_job_in_a_mix_keeps_every_image(cuda_device):
    """A job with a finite Doppler band makes its launches use the zero-window-skipping kernel
    instance; every job of the mix still gets its alone image bit for bit."""
    from sarlabtdc.serving import FocusServer

    jobs = _jobs()[:4]
    band = scenes.small_scene(seed=14, n_pri=400, n_samples=64, nx=48, ny=24, rail_len=0.4, device="cuda")
    vel = np.zeros((band.n_pri, 3), np.float32)
    vel[:, 0] = 0.05
    band_start = (0.0, 12.0, False, False, True)

    def submit_band(srv):
        return srv.submit(band.raw, band.radar.sample_times(), band.positions, band.grid,
                          np.float32(band.radar.mod_rate), np.float32(band.radar.f0), velocity=vel,
                          start=band_start)

    with FocusServer(max_jobs=6) as srv:
        alone = [srv.wait(_submit(srv, sc))[0] for sc in jobs]
        band_alone = srv.wait(submit_band(srv))[0]
        ids = [_submit(srv, sc) for sc in jobs]
        bid = submit_band(srv)
        mixed = [srv.wait(i)[0] for i in ids]
        band_mixed = srv.wait(bid)[0]
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(a, m)
    np.testing.assert_array_equal(band_alone, band_mixed)
    assert np.abs(band_alone).max() > 0


def test_many_small_jobs_from_several_client_threads(cuda_device):
    """Four client threads submit and wait on 400 small jobs in an interleaved order; every
    image equals the processor's image of the same job bit for bit."""
    import threading

    import _sarlabtdc
    from sarlabtdc.serving import FocusServer

    base = [scenes.small_scene(seed=200 + k, n_pri=64 + 16 * k, n_samples=32 + 8 * k, nx=16 + k, ny=12,
                               device="cuda") for k in range(6)]
    ref = []
    for sc in base:
        p = _sarlabtdc.TdcProcessor(0)
        p.setRawData(*sc.api_arrays().values())
        p.setChirpPositionsF64(sc.positions)
        p.setFocusGridF64(sc.grid)
        p.start(*START)
        ref.append(p.getFocusedImage().ravel().copy())
    bad, errors = [], []

    def client(tid, srv):
        try:
            rng = np.random.default_rng(tid)
            pending = []
            for _ in range(100):
                k = int(rng.integers(len(base)))
                pending.append((_submit(srv, base[k]), k))
                if rng.random() < 0.3:
                    j, kk = pending.pop(0)
                    if not np.array_equal(srv.wait(j)[0], ref[kk]):
                        bad.append(j)
            for j, kk in pending:
                if not np.array_equal(srv.wait(j)[0], ref[kk]):
                    bad.append(j)
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    with FocusServer(max_jobs=8) as srv:
        ths = [threading.Thread(target=client, args=(t, srv)) for t in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        st = srv.stats()
    assert not errors, errors
    assert not bad
    assert st["jobs_done"] == 400 and st["jobs_failed"] == 0
