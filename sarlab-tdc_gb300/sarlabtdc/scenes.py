"""Seeded synthetic FMCW scenes for the focus engine (no dataset is involved).

Beat model, in the reference's sign convention: the processor correlates
``raw * conj(ref)`` with ``ref = exp(-j 4 pi R f / c)`` (tdc-lib/src/tdckernels.cu:
202-216, 266-273), so a point target at range R focuses when

    raw[c, s] = sum_i a_i exp(-j 2 pi (f0 tau_i + K tau_i t_s - K tau_i^2 / 2)),  tau_i = 2 R_ci / c.

This is the conjugate of the usual de-chirped beat exp(+j 2 pi (...)); the residual
video phase term -K tau^2 / 2 is kept although the processor does not model it.
Raw data are computed in FP64 (torch, on the CPU or a CUDA device) and stored as
complex64, the engine's input type.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C0 = 299792458.0


@dataclass
class Radar:
    f0: float = 77e9            # chirp start frequency [Hz]
    bandwidth: float = 4e9      # swept bandwidth [Hz]
    chirp_s: float = 40e-6      # chirp duration [s]
    n_samples: int = 512

    @property
    def mod_rate(self) -> float:
        return self.bandwidth / self.chirp_s

    def sample_times(self) -> np.ndarray:
        return (np.arange(self.n_samples, dtype=np.float64) * (self.chirp_s / self.n_samples)).astype(np.float32)


@dataclass
class Scene:
    name: str
    radar: Radar
    positions: np.ndarray          # [C, 3] float64 antenna phase centres
    grid: np.ndarray               # [R, Cc, 3] float64 focus points
    targets: np.ndarray            # [N, 3] float64
    amps: np.ndarray               # [N] complex128
    raw: np.ndarray | None = None  # [C, S] complex64
    noise_sigma: float = 0.0
    hann: bool = True
    meta: dict = field(default_factory=dict)

    @property
    def n_pri(self) -> int:
        return self.positions.shape[0]

    @property
    def n_samples(self) -> int:
        return self.radar.n_samples

    @property
    def n_pix(self) -> int:
        return int(np.prod(self.grid.shape[:-1]))

    def correlations(self) -> int:
        return self.n_pix * self.n_pri * self.n_samples

    def api_arrays(self):
        """The reference API's setRawData arguments (FP32, per-sample trajectory, zero velocity,
        identity attitude, boresight +y)."""
        C, S = self.n_pri, self.n_samples
        pos = np.ascontiguousarray(np.broadcast_to(self.positions.astype(np.float32)[:, None, :], (C, S, 3)))
        vel = np.zeros((C, S, 3), dtype=np.float32)
        att = np.zeros((C, S, 4), dtype=np.float32)
        att[..., 0] = 1.0
        pri = (np.arange(C, dtype=np.float64) * 1e-3).astype(np.float32)
        return dict(rawData=self.raw, priTimes=pri, sampleTimes=self.radar.sample_times(), position=pos,
                    velocity=vel, attitude=att, modRate=np.float32(self.radar.mod_rate),
                    startFreq=np.float32(self.radar.f0), bodyBoresight=np.array([0, 1, 0], np.float32))


def hann_periodic(n: int) -> np.ndarray:
    return 0.5 - 0.5 * np.cos(2.0 * np.pi * np.arange(n) / n)


def simulate_raw(positions, targets, amps, radar: Radar, device="cpu", chunk_elems=1 << 24) -> np.ndarray:
    """FP64 beat signal [C, S] (complex128 numpy) of point targets, computed with torch."""
    import torch

    dev = torch.device(device)
    pos = torch.as_tensor(np.asarray(positions, np.float64), device=dev)
    tgt = torch.as_tensor(np.asarray(targets, np.float64), device=dev)
    amp = torch.as_tensor(np.asarray(amps, np.complex128), device=dev)
    t = torch.as_tensor(radar.sample_times().astype(np.float64), device=dev)
    C, S, N = pos.shape[0], t.shape[0], tgt.shape[0]
    out = torch.zeros((C, S), dtype=torch.complex128, device=dev)
    if N == 0:
        return out.cpu().numpy()
    cb = max(1, int(chunk_elems // max(1, N * S)))
    K = radar.mod_rate
    for c0 in range(0, C, cb):
        c1 = min(C, c0 + cb)
        R = torch.cdist(pos[c0:c1], tgt)                       # [cb, N]
        tau = 2.0 * R / C0
        base = radar.f0 * tau - 0.5 * K * tau * tau           # cycles
        base = base - torch.round(base)
        slope = K * tau                                       # cycles per second
        ph = base[:, :, None] + slope[:, :, None] * t[None, None, :]
        ph = ph - torch.round(ph)
        ang = -2.0 * math.pi * ph
        ph_c = torch.polar(torch.ones_like(ang), ang)
        out[c0:c1] = (ph_c * amp[None, :, None]).sum(dim=1)
    return out.cpu().numpy()


def finish_raw(scene: Scene, signal: np.ndarray, snr_db: float | None, rng: np.random.Generator) -> None:
    raw = signal.astype(np.complex128)
    if snr_db is not None:
        p_sig = float(np.mean(np.abs(scene.amps) ** 2)) if scene.amps.size else 1.0
        sigma = math.sqrt(p_sig / 10 ** (snr_db / 10.0))
        scene.noise_sigma = sigma
        raw = raw + sigma / math.sqrt(2.0) * (rng.standard_normal(raw.shape) + 1j * rng.standard_normal(raw.shape))
    if scene.hann:
        raw = raw * hann_periodic(raw.shape[1])[None, :]
    scene.raw = raw.astype(np.complex64)


def ground_grid(nx: int, ny: int, dx: float, y0: float, z: float = 0.0) -> np.ndarray:
    xs = (np.arange(nx) - (nx - 1) / 2.0) * dx
    ys = y0 + np.arange(ny) * dx
    g = np.zeros((ny, nx, 3), dtype=np.float64)
    g[..., 0] = xs[None, :]
    g[..., 1] = ys[:, None]
    g[..., 2] = z
    return g


def rail(n: int, length: float, height: float) -> np.ndarray:
    pos = np.zeros((n, 3), dtype=np.float64)
    pos[:, 0] = (np.arange(n) - (n - 1) / 2.0) * (length / n)
    pos[:, 2] = height
    return pos


def stripmap(seed=1, device="cpu", n_pix_side=256, n_pri=1024, n_samples=512, simulate=True) -> Scene:
    """Plain TDC stripmap: 512 samples, 1024 chirps on a 0.5 m rail (0.5 mm), 0.3 m above
    a 256 x 256 ground grid at 2 mm; 3 unit targets; 20 dB SNR; Hann."""
    rng = np.random.default_rng(seed)
    radar = Radar(n_samples=n_samples)
    pos = rail(n_pri, n_pri * 0.5e-3, 0.3)
    grid = ground_grid(n_pix_side, n_pix_side, 2e-3, y0=0.1)
    lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
    tg = np.zeros((3, 3))
    tg[:, 0] = rng.uniform(lo[0], hi[0], 3)
    tg[:, 1] = rng.uniform(lo[1], hi[1], 3)
    sc = Scene("stripmap", radar, pos, grid, tg, np.ones(3, np.complex128))
    if simulate:
        finish_raw(sc, simulate_raw(pos, tg, sc.amps, radar, device), 20.0, rng)
    return sc


def precision_study(seed=2, device="cpu", n_pix_side=1024, n_pri=4096, n_samples=1024, n_targets=50,
            simulate=True) -> Scene:
    """Precision study: 1024 samples, 4096 chirps over 2 m with 0.5 mm/axis jitter (FP64
    positions), 1024 x 1024 grid at 1 mm, 50 Rayleigh targets."""
    rng = np.random.default_rng(seed)
    radar = Radar(n_samples=n_samples)
    pos = rail(n_pri, 2.0, 0.3) + rng.normal(0.0, 0.5e-3, (n_pri, 3))
    grid = ground_grid(n_pix_side, n_pix_side, 1e-3, y0=0.2)
    lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
    tg = np.zeros((n_targets, 3))
    tg[:, 0] = rng.uniform(lo[0], hi[0], n_targets)
    tg[:, 1] = rng.uniform(lo[1], hi[1], n_targets)
    amps = rng.rayleigh(1.0, n_targets) * np.exp(2j * np.pi * rng.uniform(0, 1, n_targets))
    sc = Scene("precision_study", radar, pos, grid, tg, amps)
    if simulate:
        finish_raw(sc, simulate_raw(pos, tg, amps, radar, device), 20.0, rng)
    return sc


def volume_3d(seed=3, device="cpu", nx=256, nz=256, ny=64, n_ap=128, n_samples=256, n_targets=200,
            simulate=True) -> Scene:
    """3-D near field: 128 x 128 planar aperture at 1 mm (x-z plane, y = 0), 256 samples,
    256 x 256 x 64 voxels (1 mm lateral, 2 mm depth from 0.2 m), 200 scatterers, 15 dB."""
    rng = np.random.default_rng(seed)
    radar = Radar(n_samples=n_samples)
    ax = (np.arange(n_ap) - (n_ap - 1) / 2.0) * 1e-3
    pos = np.zeros((n_ap * n_ap, 3))
    pos[:, 0] = np.repeat(ax, n_ap)
    pos[:, 2] = np.tile(ax, n_ap)
    xs = (np.arange(nx) - (nx - 1) / 2.0) * 1e-3
    zs = (np.arange(nz) - (nz - 1) / 2.0) * 1e-3
    ys = 0.2 + np.arange(ny) * 2e-3
    # R x C = (depth * z) x x, row-major: voxel (iy, iz, ix)
    g = np.zeros((ny, nz, nx, 3))
    g[..., 0] = xs[None, None, :]
    g[..., 1] = ys[:, None, None]
    g[..., 2] = zs[None, :, None]
    grid = g.reshape(ny * nz, nx, 3)
    tg = np.stack([rng.uniform(xs[0], xs[-1], n_targets), rng.uniform(ys[0], ys[-1], n_targets),
                   rng.uniform(zs[0], zs[-1], n_targets)], axis=1)
    amps = np.exp(2j * np.pi * rng.uniform(0, 1, n_targets))
    sc = Scene("volume_3d", radar, pos, grid, tg, amps)
    if simulate:
        finish_raw(sc, simulate_raw(pos, tg, amps, radar, device), 15.0, rng)
    return sc


def autofocus_scene(seed=5, device="cpu", n_pix_side=512, n_pri=4096, n_samples=1024, n_targets=30,
            step_sigma=0.2e-3, simulate=True) -> Scene:
    """Autofocus: 4096 chirps x 1024 samples over 2 m, true trajectory = nominal rail + a
    random walk (0.2 mm per step per axis); 512 x 512 grid at 1 mm; 30 targets.
    ``positions`` is the nominal (what the processor is told); the walk is in meta."""
    rng = np.random.default_rng(seed)
    radar = Radar(n_samples=n_samples)
    nominal = rail(n_pri, 2.0, 0.3)
    walk = np.cumsum(rng.normal(0.0, step_sigma, (n_pri, 3)), axis=0)
    walk -= walk.mean(axis=0, keepdims=True)
    true_pos = nominal + walk
    grid = ground_grid(n_pix_side, n_pix_side, 1e-3, y0=0.3)
    lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
    tg = np.zeros((n_targets, 3))
    tg[:, 0] = rng.uniform(lo[0], hi[0], n_targets)
    tg[:, 1] = rng.uniform(lo[1], hi[1], n_targets)
    amps = rng.rayleigh(1.0, n_targets) * np.exp(2j * np.pi * rng.uniform(0, 1, n_targets))
    sc = Scene("autofocus_scene", radar, nominal, grid, tg, amps, meta={"walk": walk, "true_positions": true_pos})
    if simulate:
        finish_raw(sc, simulate_raw(true_pos, tg, amps, radar, device), 20.0, rng)
    return sc


def small_scene(seed=0, n_pri=256, n_samples=128, nx=24, ny=20, n_targets=3, jitter=0.0, snr_db=20.0,
                device="cpu", rail_len=None, spacing=2e-3, y0=0.12, height=0.3) -> Scene:
    """A stripmap scene (rail above a ground grid) small enough for an FP64 CPU check in a test."""
    rng = np.random.default_rng(seed)
    radar = Radar(n_samples=n_samples)
    pos = rail(n_pri, rail_len if rail_len is not None else n_pri * 0.5e-3, height)
    if jitter:
        pos = pos + rng.normal(0.0, jitter, pos.shape)
    grid = ground_grid(nx, ny, spacing, y0=y0)
    lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
    tg = np.zeros((n_targets, 3))
    tg[:, 0] = rng.uniform(lo[0], hi[0], n_targets)
    tg[:, 1] = rng.uniform(lo[1], hi[1], n_targets)
    amps = np.exp(2j * np.pi * rng.uniform(0, 1, n_targets))
    sc = Scene("small", radar, pos, grid, tg, amps)
    finish_raw(sc, simulate_raw(pos, tg, amps, radar, device), snr_db, rng)
    return sc
