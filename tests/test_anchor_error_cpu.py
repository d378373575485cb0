"""CPU check of the error bound of anchored ranges: the range difference from an anchor,
dR = d.(d - 2e) / (R0 + R) with d = pixel - anchor and e = antenna - anchor, formed in FP32
(numpy float32 with the kernel's fused multiply-adds) as the anchored focus kernel forms it,
against the FP64 range, keeps the two-way phase at 77 GHz within 4e-5 rad for pixels up to
the 5 cm anchor bound and within 1.5e-5 rad up to 1.6 cm (32 pixels of a 1 mm grid), over
near-field (3-D volume) and stripmap geometries."""
import math

import numpy as np

C0 = 299792458.0
F0 = 77e9


def _anchored_phase_error(ant, pix, anchor):
    f32 = np.float32
    e64 = ant[:, None, :] - anchor[None, :, :]
    R0 = np.linalg.norm(e64, axis=-1)
    e = e64.astype(f32)
    d = (pix - anchor).astype(f32)[None]
    r = lambda x: np.asarray(x, dtype=f32)  # noqa: E731  (one FP32 rounding)

    def fma(a, b, c):  # FP32 fused multiply-add: the exact product in FP64, one rounding
        return r(a.astype(np.float64) * b.astype(np.float64) + np.asarray(c, np.float64))

    u = [r(d[..., k] - f32(2) * e[..., k]) for k in range(3)]  # fmaf(-2, e, d): 2e is exact
    num = r(d[..., 0] * u[0])
    num = fma(d[..., 1], u[1], num)
    num = fma(d[..., 2], u[2], num)
    dv = r(e - d)
    r2 = fma(dv[..., 0], dv[..., 0], fma(dv[..., 1], dv[..., 1], r(dv[..., 2] * dv[..., 2])))
    rr = r(np.sqrt(r2))
    dR = r(num / r(R0.astype(f32) + rr))
    true = np.linalg.norm(ant[:, None, :] - pix[None, :, :], axis=-1)
    return 2.0 * math.pi * 2.0 * F0 / C0 * np.abs(R0 + dR.astype(np.float64) - true)


def test_anchored_range_phase_error_within_bound():
    for dmax, bound in ((0.05, 4e-5), (0.016, 1.5e-5)):
        worst = _worst(dmax)
        assert worst <= bound, (dmax, worst)


def _worst(dmax):
    rng = np.random.default_rng(11)
    worst = 0.0
    # stripmap: 2 m rail 0.3 m above the grid; 3-D volume: 128 mm planar aperture, voxels from 0.2 m
    rail = np.stack([np.linspace(-1.0, 1.0, 257), np.zeros(257), np.full(257, 0.3)], 1)
    ap = (np.stack(np.meshgrid(np.arange(16), np.arange(16)), -1).reshape(-1, 2) * 8e-3 - 0.064)
    plane = np.stack([ap[:, 0], np.zeros(len(ap)), ap[:, 1]], 1)
    for ant, lo, hi in ((rail, (-0.5, 0.2, 0.0), (0.5, 1.2, 0.0)), (plane, (-0.13, 0.2, -0.13), (0.13, 0.33, 0.13))):
        anchor = rng.uniform(lo, hi, (400, 3))
        direction = rng.normal(size=(400, 3))
        direction /= np.linalg.norm(direction, axis=1, keepdims=True)
        pix = anchor + direction * rng.uniform(0.0, dmax, (400, 1))
        err = _anchored_phase_error(ant, pix, anchor)
        worst = max(worst, float(err.max()))
    return worst
