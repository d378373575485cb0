"""GPU tests of the focus adjoint (autofocus): against the FP64 oracle's gradient,
against central finite differences of the engine's own forward, through
torch.autograd with the entropy loss, and one short autofocus run."""
import numpy as np
import pytest

import oracle
from sarlabtdc import scenes

pytestmark = pytest.mark.gpu

INF = float("inf")
ARGS = (0.0, INF, False, False, True)


def _operator(sc):
    import _sarlabtdc
    from sarlabtdc import autofocus

    api = sc.api_arrays()
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setChirpPositionsF64(sc.positions)
    p.setFocusGridF64(sc.grid)
    return autofocus.FocusOperator(p, ARGS), api


def _loss_linear(img, g):
    return float(np.real(np.sum(np.conj(g) * img)))


def test_adjoint_matches_oracle_gradient(cuda_device):
    import torch

    sc = scenes.small_scene(seed=71, n_pri=96, n_samples=64, nx=16, ny=14, jitter=0.2e-3, device="cuda")
    op, api = _operator(sc)
    rng = np.random.default_rng(5)
    off = rng.normal(0, 0.1e-3, (sc.n_pri, 3))
    g = (rng.normal(size=op.n_pix) + 1j * rng.normal(size=op.n_pix)).astype(np.complex64)
    got = op.adjoint(torch.from_numpy(off).cuda(), torch.from_numpy(g).cuda()).cpu().numpy()
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid)
    ref = oracle.adjoint_offsets(prob, oracle.Opts(), off, g.astype(np.complex128))
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 1e-3, err
    np.testing.assert_allclose(got, ref, rtol=2e-2, atol=2e-3 * np.abs(ref).max())


def test_adjoint_matches_finite_differences_of_the_forward(cuda_device):
    import torch

    sc = scenes.small_scene(seed=72, n_pri=64, n_samples=64, nx=12, ny=12, device="cuda")
    op, _ = _operator(sc)
    rng = np.random.default_rng(6)
    g = (rng.normal(size=op.n_pix) + 1j * rng.normal(size=op.n_pix)).astype(np.complex64)
    off = torch.from_numpy(rng.normal(0, 0.05e-3, (sc.n_pri, 3))).cuda()
    grad = op.adjoint(off, torch.from_numpy(g).cuda()).cpu().numpy()
    h = 1e-5   # FP32 forward: a larger step than the FP64 oracle's 1e-6 keeps rounding out of the difference
    for c, k in [(0, 0), (17, 1), (40, 2), (63, 1)]:
        e = torch.zeros_like(off)
        e[c, k] = h
        lp = _loss_linear(op.image(off + e).cpu().numpy(), g)
        lm = _loss_linear(op.image(off - e).cpu().numpy(), g)
        fd = (lp - lm) / (2 * h)
        assert grad[c, k] == pytest.approx(fd, rel=2e-2, abs=2e-3 * np.abs(grad).max())


def test_autograd_entropy_gradient(cuda_device):
    import torch
    from sarlabtdc import autofocus

    sc = scenes.small_scene(seed=73, n_pri=64, n_samples=64, nx=14, ny=12, device="cuda")
    op, _ = _operator(sc)
    x = torch.zeros((sc.n_pri, 3), dtype=torch.float64, device="cuda", requires_grad=True)
    loss = autofocus.entropy(autofocus.focus(op, x))
    loss.backward()
    h = 1e-5
    for c, k in [(3, 0), (30, 1), (50, 2)]:
        e = torch.zeros_like(x)
        e[c, k] = h
        with torch.no_grad():
            lp = float(autofocus.entropy(op.image(x + e)))
            lm = float(autofocus.entropy(op.image(x - e)))
        fd = (lp - lm) / (2 * h)
        assert float(x.grad[c, k]) == pytest.approx(fd, rel=3e-2, abs=3e-3 * float(x.grad.abs().max()))


def test_autofocus_descends_the_entropy(cuda_device):
    """The Adam loop over the autograd Function lowers the objective. (Whether the entropy
    minimum is the true trajectory depends on the scene: with free per-chirp 3-D offsets it
    can over-sharpen; bench.py --config 5 reports the coherence with the true-trajectory image.)"""
    import torch
    from sarlabtdc import autofocus

    rng = np.random.default_rng(8)
    sc = scenes.small_scene(seed=74, n_pri=128, n_samples=64, nx=24, ny=24, n_targets=6, device="cuda")
    walk = np.cumsum(rng.normal(0, 0.05e-3, (sc.n_pri, 3)), axis=0)
    walk -= walk.mean(0)
    scenes.finish_raw(sc, scenes.simulate_raw(sc.positions + walk, sc.targets, sc.amps, sc.radar, "cuda"), 30.0, rng)
    op, _ = _operator(sc)
    res = autofocus.autofocus(op, steps=20, lr=1e-5)
    assert res.entropy[-1] < res.entropy[0]
    assert np.all(np.isfinite(res.offsets.cpu().numpy()))
    assert len(res.step_ms) == 20


@pytest.mark.parametrize("band", [INF, 14.0])
def test_adjoint_with_kept_sums_matches_recomputation(cuda_device, band):
    """A forward that keeps its per-chirp sums lets the adjoint compute only the
    index-weighted sums from rows pre-scaled by the sample index; its gradient matches the
    full recomputation and the FP64 oracle's, with an unbounded band and a finite one (the
    antenna moving along the rail: chirps the window vote skips keep zero sums). A
    trajectory change between forward and adjoint makes the kept sums stale: the adjoint
    recomputes."""
    import torch

    import _sarlabtdc
    from sarlabtdc import autofocus

    sc = scenes.small_scene(seed=73, n_pri=160, n_samples=64, nx=40, ny=35, jitter=0.2e-3, rail_len=0.4,
                            device="cuda")
    api = sc.api_arrays()
    vel = np.zeros((sc.n_pri, sc.n_samples, 3), np.float32)
    vel[..., 0] = 0.08
    api["velocity"] = vel
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setChirpPositionsF64(sc.positions)
    p.setFocusGridF64(sc.grid)
    args = (0.0, band, False, False, True)
    op = autofocus.FocusOperator(p, args)
    rng = np.random.default_rng(8)
    off = torch.from_numpy(rng.normal(0, 0.1e-3, (sc.n_pri, 3))).cuda()
    g = torch.from_numpy((rng.normal(size=op.n_pix) + 1j * rng.normal(size=op.n_pix)).astype(np.complex64)).cuda()

    op.image(off)
    kept = op.adjoint(off, g).cpu().numpy()
    assert p.lastStats()["adjoint_stored"] == 1
    p.keepChirpSums(False)
    full = op.adjoint(off, g).cpu().numpy()
    assert p.lastStats()["adjoint_stored"] == 0
    assert np.linalg.norm(kept - full) / np.linalg.norm(full) < 1e-4

    if not np.isfinite(band):
        # (under a finite band FP32 and FP64 can put a (pixel, chirp) on either side of the
        # band edge; there the two engine paths are compared with each other only)
        prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                              velocity=vel[:, 0, :], modRate=api["modRate"], startFreq=api["startFreq"],
                              grid=sc.grid)
        ref = oracle.adjoint_offsets(prob, oracle.Opts(), off.cpu().numpy(), g.cpu().numpy().astype(np.complex128))
        assert np.linalg.norm(kept - ref) / np.linalg.norm(ref) < 1e-3

    # stale sums: a forward at the old offsets, then the adjoint at new ones
    p.keepChirpSums(True)
    op.image(off)
    off2 = off + torch.from_numpy(rng.normal(0, 0.05e-3, (sc.n_pri, 3))).cuda()
    at2 = op.adjoint(off2, g).cpu().numpy()
    assert p.lastStats()["adjoint_stored"] == 0
    p.keepChirpSums(False)
    at2_full = op.adjoint(off2, g).cpu().numpy()
    np.testing.assert_array_equal(at2, at2_full)
