"""Autofocus through the focus adjoint (no reference counterpart).

The focused image is a differentiable function of per-chirp antenna-position
offsets d_c (metres, FP64): ``focus(op, offsets)`` is a torch.autograd.Function
whose forward is the FP32-bulk focus kernel on the offset trajectory and whose
backward is the hand-written adjoint kernel (tdc_processor_adjoint_device):

    dL/dd_c = sum_p Re(conj(G_p) dI_p/dR_pc) (P_c + d_c - T_p) / R_pc,

G = dL/dRe I + j dL/dIm I (torch's gradient of a complex tensor). The Doppler
window and skip test are held fixed. ``autofocus`` minimises the image entropy
of |I|^2 with Adam, over free per-chirp offsets or over a smooth correction to a
starting trajectory (a piecewise-linear basis of control points along the chirps,
``hat_basis``; its gradient is the adjoint's, chained through the basis by autograd).

The entropy's basin around the true trajectory is narrow: on the benchmark's
random walk (6.4 mm RMS, 1.7 wavelengths) the true offsets are a local minimum, and a
start from a smooth estimate of them (the walk averaged over ~32 mm of rail)
converges to the focused image with a 256-point basis, but Adam from the nominal
trajectory does not reach it (the entropy then falls below the focused image's by
sharpening a wrong image).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

import _sarlabtdc


class FocusOperator:
    """A processor with its acquisition and grid resident on the device."""

    def __init__(self, proc: _sarlabtdc.TdcProcessor, start_args=(0.0, float("inf"), False, False, True),
                 keep_sums: bool = True):
        self.proc = proc
        proc.prepare(*start_args)
        proc.uploadGrid()
        if proc.path() != "fp32_bulk":
            raise RuntimeError("autofocus needs the FP32-bulk path (per-chirp trajectory, uniform sampling)")
        self.n_pix = proc.numPixels()
        self.n_pri = proc.numChirps()
        # the forward keeps its per-chirp sums, so the adjoint recomputes only half
        proc.keepChirpSums(keep_sums)
        self._offsets = None  # offsets the resident trajectory was last set to

    def _set_offsets(self, offsets: torch.Tensor | None):
        o = None if offsets is None else offsets.detach().contiguous()
        same = (o is None and self._offsets is None) or (
            o is not None and self._offsets is not None and torch.equal(o, self._offsets))
        if not same:
            self.proc.setChirpOffsetsDevice(o)
            self._offsets = None if o is None else o.clone()

    def image(self, offsets: torch.Tensor | None) -> torch.Tensor:
        self._set_offsets(offsets)
        img = torch.empty(self.n_pix, dtype=torch.complex64, device="cuda")
        self.proc.focusDevice(img)
        return img

    def adjoint(self, offsets: torch.Tensor, grad_image: torch.Tensor) -> torch.Tensor:
        # the forward's offsets are usually still set: the kept sums then stay valid
        self._set_offsets(offsets)
        g = torch.empty((self.n_pri, 3), dtype=torch.float64, device="cuda")
        self.proc.adjointDevice(grad_image.detach().to(torch.complex64).contiguous(), g)
        return g


class _Focus(torch.autograd.Function):
    @staticmethod
    def forward(ctx, offsets, op):
        ctx.op = op
        ctx.save_for_backward(offsets.detach().clone())
        return op.image(offsets)

    @staticmethod
    def backward(ctx, grad_image):
        (offsets,) = ctx.saved_tensors
        return ctx.op.adjoint(offsets, grad_image), None


def focus(op: FocusOperator, offsets: torch.Tensor) -> torch.Tensor:
    """Differentiable focus: complex64 image [n_pix] of the trajectory base + offsets [n_pri, 3]."""
    return _Focus.apply(offsets, op)


def entropy(img: torch.Tensor) -> torch.Tensor:
    """Shannon entropy of the normalised intensity |I|^2 / sum |I|^2."""
    inten = img.real.double() ** 2 + img.imag.double() ** 2
    p = inten / inten.sum()
    return -(p * torch.log(p + 1e-300)).sum()


@dataclass
class AutofocusResult:
    offsets: torch.Tensor
    entropy: list = field(default_factory=list)
    step_ms: list = field(default_factory=list)


def hat_basis(n_chirps: int, knots: int, device="cuda") -> torch.Tensor:
    """[n_chirps, knots] FP64 piecewise-linear interpolation from `knots` control points spread
    evenly over the chirps (each column a hat function; rows sum to 1)."""
    if knots < 2 or knots > n_chirps:
        raise ValueError("knots must be between 2 and the number of chirps")
    x = torch.arange(n_chirps, dtype=torch.float64) * ((knots - 1) / max(1, n_chirps - 1))
    i0 = torch.clamp(torch.floor(x).long(), 0, knots - 2)
    f = x - i0
    B = torch.zeros((n_chirps, knots), dtype=torch.float64)
    rows = torch.arange(n_chirps)
    B[rows, i0] = 1.0 - f
    B[rows, i0 + 1] = f
    return B.to(device)


def autofocus(op: FocusOperator, steps: int = 50, lr: float = 2e-5, offsets: torch.Tensor | None = None,
              knots: int | None = None, callback=None) -> AutofocusResult:
    """Minimise image entropy with Adam; returns the offsets and the entropy history.

    ``offsets`` [n_pri, 3] is the starting trajectory correction (zero by default). With
    ``knots`` the parameters are a smooth correction to it, offsets + B theta with B =
    hat_basis(n_pri, knots) and theta starting at zero; without, the offsets themselves."""
    if offsets is None:
        offsets = torch.zeros((op.n_pri, 3), dtype=torch.float64, device="cuda")
    base = offsets.detach().to(torch.float64)
    B = None
    if knots:
        B = hat_basis(op.n_pri, int(knots), base.device)
        theta = torch.zeros((B.shape[1], 3), dtype=torch.float64, device=base.device, requires_grad=True)
    else:
        theta = base.clone().requires_grad_(True)

    def trajectory():
        return theta if B is None else base + B @ theta

    opt = torch.optim.Adam([theta], lr=lr)
    res = AutofocusResult(offsets=theta)
    for it in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        opt.zero_grad()
        loss = entropy(focus(op, trajectory()))
        loss.backward()
        opt.step()
        e1.record()
        torch.cuda.synchronize()
        res.entropy.append(float(loss.detach()))
        res.step_ms.append(e0.elapsed_time(e1))
        if callback:
            callback(it, res)
    with torch.no_grad():
        x = trajectory().detach()
        res.entropy.append(float(entropy(op.image(x))))
    res.offsets = x
    return res


def coherence(a, b) -> float:
    """|<a, b>| / (|a| |b|): 1 when two images agree up to a common complex factor."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b)))


def residual_phase_rms(offsets_est: np.ndarray, offsets_true: np.ndarray, positions: np.ndarray,
                       centre: np.ndarray, wavelength: float) -> float:
    """RMS over chirps of the two-way phase error 4 pi / lambda * u_c . (true - estimate) towards the scene
    centre, after removing its mean (a common shift only translates the image)."""
    u = centre[None, :] - positions
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    err = 4.0 * math.pi / wavelength * np.einsum("ij,ij->i", -u, offsets_true - offsets_est)
    err -= err.mean()
    return float(np.sqrt(np.mean(err ** 2)))
