"""Compile-time tuning sweep of the FP32-bulk focus kernel.

Each variant is the engine rebuilt with extra ``-D`` flags (the kernel's knobs:
TDC_FOCUS_L, TDC_FOCUS_PT, TDC_FOCUS_MINB, TDC_FOCUS_UNROLL, TDC_FOCUS_SWAP,
TDC_FOCUS_STAGE_TARGET) into ``_build/variants/<name>/``, then timed on three
synthetic shapes with the acquisition and grid resident on the device:

    2: 1024^2 pixels x 4096 chirps x 1024 samples (the precision-study size)
    3: 1024^2 pixels x 4096 chirps x  256 samples (the 3-D volume's sample count)
    1: 256^2 pixels x 1024 chirps x 512 samples (the small stripmap case)
    2b: shape 2 with the antenna moving at 0.05 m/s along the rail and a 10 Hz Doppler
        band (windowed focus: zero-window chirps skipped)

and, for the general kernel (TDC_GENERAL_PT, TDC_GENERAL_MINB, TDC_GENERAL_STAGE_TARGET,
TDC_GENERAL_ALWAYS_SEGMENT),
on 512^2 pixels x 1024 chirps x 1024 samples with FP32 per-sample inputs:

    g:  positions drifting ~0.3 mm within each chirp
    gw: the same plus per-sample velocity under a 30 Hz Doppler band
    gn: jittered (non-uniform) sample times
    gl: positions as g on long chirps, 256^2 pixels x 256 chirps x 4096 samples (rows
        staged in segments)
    gs: positions as g on a small aperture, 256^2 pixels x 256 chirps x 1024 samples

Timing: 2 warm-up focuses, then the mean of 3 focuses between CUDA events on the
launching stream. Each variant's image is compared with the first variant's.

    python sarlab-tdc_gb300/tune_focus.py base= u4=-DTDC_FOCUS_UNROLL=4 "s4=-DTDC_FOCUS_SWAP=1 -DTDC_FOCUS_UNROLL=4"
    python sarlab-tdc_gb300/tune_focus.py --shapes g,gw,gn base= "pt2=-DTDC_GENERAL_PT=2 -DTDC_GENERAL_MINB=2"
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

PKG = Path(__file__).resolve().parent
SHAPES = ("2", "3", "1")


def _time_shape(shape: str, ref_dir: Path) -> dict:
    sys.path.insert(0, str(PKG))
    import numpy as np
    import torch

    import _sarlabtdc
    from sarlabtdc import scenes

    band = float("inf")
    if shape == "1":
        sc = scenes.stripmap(device="cuda")
    elif shape in ("gl", "gs"):
        sc = scenes.precision_study(device="cuda", n_pix_side=256, n_pri=256, n_samples=4096 if shape == "gl" else 1024,
                            n_targets=8)
    elif shape.startswith("g"):
        sc = scenes.precision_study(device="cuda", n_pix_side=512, n_pri=1024, n_samples=1024, n_targets=8)
    else:
        sc = scenes.precision_study(device="cuda", n_pix_side=1024, n_pri=4096, n_samples=256 if shape == "3" else 1024,
                            n_targets=8)
    api = sc.api_arrays()
    if shape == "2b":
        vel = np.zeros((sc.n_pri, sc.n_samples, 3), np.float32)
        vel[..., 0] = 0.05
        api["velocity"] = vel
        band = 10.0
    p = _sarlabtdc.TdcProcessor(0)
    if shape.startswith("g"):
        C, S = sc.n_pri, sc.n_samples
        rng = np.random.default_rng(1)
        if shape in ("g", "gw", "gl", "gs"):
            pos = np.broadcast_to(sc.positions[:, None, :], (C, S, 3)) + \
                (np.arange(S) / S)[None, :, None] * rng.normal(0.0, 0.3e-3, (C, 1, 3))
            api["position"] = np.ascontiguousarray(pos, dtype=np.float32)
        if shape == "gw":
            vel = np.zeros((C, S, 3), np.float32)
            vel[..., 0] = 0.05 + 0.01 * np.sin(np.arange(S) / 7.0)[None, :]
            api["velocity"] = vel
            band = 30.0
        if shape == "gn":
            st = api["sampleTimes"].astype(np.float64)
            st += rng.uniform(-0.3, 0.3, st.shape) * (st[1] - st[0])
            api["sampleTimes"] = st.astype(np.float32)
        p.setRawData(*api.values())
        p.setFocusGrid(sc.grid.astype(np.float32))
    else:
        p.setRawData(*api.values())
        p.setChirpPositionsF64(sc.positions)
        p.setFocusGridF64(sc.grid)
    p.prepare(0.0, band, False, False, True)
    p.uploadGrid()
    img = torch.empty(p.numPixels(), dtype=torch.complex64, device="cuda")
    for _ in range(2):
        p.focusDevice(img)
    p.check()
    n = 3
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(n):
        p.focusDevice(img)
    ev[1].record()
    torch.cuda.synchronize()
    p.check()
    ms = ev[0].elapsed_time(ev[1]) / n
    out = img.cpu().numpy()
    ref_f = ref_dir / f"shape_{shape}.npy"
    if not ref_f.exists():
        np.save(ref_f, out)
    ref = np.load(ref_f)
    st = p.lastStats()
    return {"ms": round(ms, 3), "gcorr_s": round(sc.correlations() / (ms / 1e3) / 1e9, 1), "path": p.path(),
            "stage": [st["stage_samples"], st["stage_chirps"]],
            "rel_vs_first": float(np.linalg.norm(out - ref) / np.linalg.norm(ref))}


def main(argv: list[str]) -> int:
    if argv[:1] == ["--time"]:
        print(json.dumps(_time_shape(argv[1], Path(argv[2]))), flush=True)
        return 0
    sys.path.insert(0, str(PKG))
    import build as engine_build

    shapes = SHAPES
    if argv[:1] == ["--shapes"]:
        shapes = tuple(argv[1].split(","))
        argv = argv[2:]
    variants = [a.split("=", 1) for a in argv] or [["base", ""]]
    ref_dir = Path(tempfile.mkdtemp(prefix="tdc_tune_"))
    for name, flags in variants:
        out_dir = engine_build.BUILD / "variants" / name
        lib = engine_build.build(defines=tuple(flags.split()), out_dir=out_dir, lib=out_dir / "libtdc_gb300.so")
        for shape in shapes:
            r = subprocess.run([sys.executable, __file__, "--time", shape, str(ref_dir)],
                               env={**os.environ, "TDC_GB300_LIB": str(lib)}, capture_output=True, text=True,
                               timeout=900)
            line = r.stdout.strip().splitlines()[-1] if r.returncode == 0 and r.stdout.strip() else \
                "failed: " + r.stderr[-400:]
            print(name, shape, line, flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
