#!/usr/bin/env python3
"""Benchmark of the GB300 TDC focus (TdcProcessor::start's hot path).

Workload: the precision study -- 1024 x 1024 pixels at 1 mm, 4096 chirps x 1024
samples over a 2 m jittered trajectory (FP64 positions and grid), 50 Rayleigh
targets + noise, seeded synthetic data. Metric: Gcorr/s (pixel x chirp x
sample correlations per second).

One JSON line on stdout:
  value     device-resident throughput of the FP32-bulk focus (inputs in HBM)
  e2e       the same metric through the processor C ABI with host buffers
            (setRawData / setFocusGrid / start: H2D, focus, D2H every step)
  roofline  focus kernel vs the measured FP32 FFMA peak (8 FLOP = one complex
            multiply-accumulate per correlation)
  cpu_baseline  the FP64 OpenMP oracle loop on the host cores, bounded sample
  plain     the all-FP64-phase comparator kernel and the speed-up over it
  general   the FP32 general kernel (per-sample trajectory) on a row band vs the FP64 one
  accuracy  engine vs the FP64 oracle on a pixel sample (rel. L2, phase, peak)

``--impl reference`` times the reference arm: the reference has no CPU focus,
so its CPU implementation of the path is the oracle's restatement (port),
with all host threads, on bounded pixel samples of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "sarlab-tdc_gb300"))

import numpy as np  # noqa: E402

METRIC = "Gcorr/s (pixel*chirp*sample) & p50/p99 focus latency vs plain @<=1e-4 L2"
UNIT = "Gcorr/s"
FLOP_PER_CORR = 8.0  # complex multiply-accumulate: 4 FFMA


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="2", choices=["1", "2", "3", "4", "5"],
                    help="1: 256^2 stripmap, 1024 x 512; 2: precision study (default); 3: 3-D volume; "
                         "4: serving mix; 5: autofocus")
    ap.add_argument("--jobs", type=int, default=256, help="config 4: number of requests")
    ap.add_argument("--rate", type=float, default=20.0, help="config 4: mean arrivals per second")
    ap.add_argument("--af-steps", type=int, default=50, help="config 5: Adam steps")
    ap.add_argument("--af-lr", type=float, default=5e-5, help="config 5: Adam learning rate [m]")
    ap.add_argument("--side", type=int, default=1024, help="grid side (pixels), config 2")
    ap.add_argument("--chirps", type=int, default=4096, help="config 2")
    ap.add_argument("--samples", type=int, default=1024, help="config 2")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--quick", action="store_true", help="skip plain / e2e / CPU / serving / autofocus legs")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-mix leg of the default run")
    ap.add_argument("--no-autofocus", action="store_true", help="skip the autofocus leg of the default run")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the oracle accuracy check")
    ap.add_argument("--general-only", action="store_true",
                    help="config 2 scene: only the FP32 vs FP64 general-kernel leg (per-sample trajectory)")
    ap.add_argument("--windowed-only", action="store_true",
                    help="config 2 scene: only the windowed leg (moving antenna, finite Doppler band)")
    return ap.parse_args()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", "0"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = max((num(r[2]) or 0) for r in rows)
        power = [num(r[3]) for r in rows if num(r[3]) is not None]
        loaded = [s for s in sm if s >= 0.5 * smax] or sm
        reasons = set()
        names = {5: "hw_slowdown", 6: "hw_thermal_slowdown", 7: "sw_thermal_slowdown", 8: "sw_power_cap"}
        for r in rows:
            for i, nm in names.items():
                if r[i].lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(loaded)) if loaded else None, "sm_max_mhz": smax,
                "power_w_max": max(power) if power else None, "samples": len(rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
WORKLOADS = {
    "1": "plain stripmap: 256x256 px @2mm, 1024 chirps x 512 samples, 0.5 m rail, FP32 API inputs",
    "3": "3-D volume: 256x256x64 voxels, 128x128 planar aperture @1mm, 256 samples, FP32 API inputs",
}


def uses_f64(args):
    return args.config == "2"


def workload(args, sc):
    if args.config == "2":
        return (f"precision study: {args.side}x{args.side} px @1mm, {sc.n_pri} chirps x {sc.n_samples} samples, "
                "2 m jittered rail, FP64 positions + grid")
    return WORKLOADS[args.config]


def bench_config(args, sc):
    """The workload record, the same object in both arms."""
    return {"workload": workload(args, sc), "pixels": sc.n_pix, "chirps": sc.n_pri, "samples": sc.n_samples,
            "l2": "GPU arm: a 256 MiB buffer is written between timed steps (L2 is 129 MB)"}


def make_scene(args, device):
    from sarlabtdc import scenes

    t = time.time()
    if args.config == "1":
        sc = scenes.stripmap(device=device)
    elif args.config == "3":
        sc = scenes.volume_3d(device=device)
    else:
        sc = scenes.precision_study(device=device, n_pix_side=args.side, n_pri=args.chirps, n_samples=args.samples)
    log(f"scene: {sc.n_pix} px x {sc.n_pri} chirps x {sc.n_samples} samples "
        f"({sc.correlations() / 1e9:.1f} Gcorr) generated in {time.time() - t:.1f}s")
    return sc


def sample_pixels(sc, n_random, seed=0):
    rng = np.random.default_rng(seed)
    flat = sc.grid.reshape(-1, 3)
    near = [int(np.argmin(np.linalg.norm(flat - t, axis=1))) for t in sc.targets]
    rnd = rng.choice(flat.shape[0], size=min(n_random, flat.shape[0]), replace=False).tolist()
    return np.array(sorted(set(near + rnd)), dtype=np.int64)


def oracle_problem(sc, api, f64=True):
    """The oracle on exactly the inputs the engine receives (FP64 trajectory and grid
    through the extensions, or the FP32 API arrays)."""
    import oracle

    if f64:
        return oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                              modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid)
    return oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=api["position"][:, 0, :],
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid.astype(np.float32))


def oracle_opts():
    import oracle

    # Hann is applied to the raw data by the generator: no range window, infinite Doppler band
    return oracle.Opts(applyRangeWin=False, dopplerBandwidth=float("inf"))


def time_oracle(sc, api, budget_s, threads, f64=True):
    """FP64 oracle throughput (Gcorr/s) on a bounded pixel sample sized to ~budget_s."""
    import oracle

    build_oracle()
    prob = oracle_problem(sc, api, f64)
    o = oracle_opts()
    rng = np.random.default_rng(123)
    per_px = sc.n_pri * sc.n_samples
    n = 16
    t = time.perf_counter()
    oracle.focus(prob, o, pixels=rng.choice(sc.n_pix, n, replace=False), threads=threads)
    dt = time.perf_counter() - t
    n2 = int(max(n, min(sc.n_pix, n * budget_s / max(dt, 1e-3))))
    pix = rng.choice(sc.n_pix, n2, replace=False)
    t = time.perf_counter()
    oracle.focus(prob, o, pixels=pix, threads=threads)
    dt = time.perf_counter() - t
    return n2 * per_px / dt / 1e9, n2, dt


def build_oracle():
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob

    ob.build_oracle()


def fp32_peak_tflops(lib, torch):
    import ctypes as C

    dev = torch.cuda.current_device()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    scratch = torch.empty(n_sm * 64 * 8, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    flops = C.c_double()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rc = lib.tdc_probe_fma(0, n_sm * 8, 1000, scratch.data_ptr(), C.byref(flops), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        assert rc == 0
        best = max(best, flops.value / (e0.elapsed_time(e1) / 1e3) / 1e12)
    fp64 = 0.0
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lib.tdc_probe_fma(1, n_sm * 2, 25, scratch.data_ptr(), C.byref(flops), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64 = max(fp64, flops.value / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best, fp64, n_sm


def load_traffic():
    f = ROOT / "profiles" / "focus_fp32_traffic.json"
    if f.exists():
        try:
            return json.loads(f.read_text())
        except ValueError:
            return None
    return None


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    import _sarlabtdc
    import _tdc_capi

    assert torch.cuda.is_available(), "bench.py needs a CUDA device"
    torch.cuda.set_device(0)
    lib = _tdc_capi.lib()
    sc = make_scene(args, "cuda")
    api = sc.api_arrays()
    P, Cn, S = sc.n_pix, sc.n_pri, sc.n_samples
    corr = sc.correlations()
    inf = float("inf")
    start_args = (0.0, inf, False, False, True)

    f64 = uses_f64(args)

    def load(proc, grid):
        proc.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                        api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
        if f64:
            proc.setChirpPositionsF64(sc.positions)
            proc.setFocusGridF64(grid)
        else:
            proc.setFocusGrid(grid.astype(np.float32))

    p = _sarlabtdc.TdcProcessor(0)
    load(p, sc.grid)
    p.prepare(*start_args)
    p.uploadGrid()
    path = p.path()
    img = torch.empty(P, dtype=torch.complex64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    stream = torch.cuda.current_stream()

    for _ in range(max(3, args.warmup)):
        p.focusDevice(img, stream)
        flush.zero_()
    p.check(stream)

    clocks = Clocks()
    clocks.start()
    time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for e0, e1 in evs:
        e0.record(stream)
        p.focusDevice(img, stream)
        e1.record(stream)
        flush.zero_()
    t1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    p.check(stream)
    total_ms = t0.elapsed_time(t1)
    step_ms = np.array([a.elapsed_time(b) for a, b in evs])
    value = corr * args.steps / (total_ms / 1e3) / 1e9
    kernel_gcorr = corr / (step_ms.mean() / 1e3) / 1e9
    log(f"value {value:.1f} Gcorr/s  focus launch {step_ms.mean():.2f} ms  path={path}  clocks={clk}")
    image = img.cpu().numpy()

    peak_tf, fp64_tf, n_sm = fp32_peak_tflops(lib, torch)
    achieved_tf = kernel_gcorr * FLOP_PER_CORR / 1e3
    traffic = load_traffic()
    roofline = {"bound": "fp32", "achieved": round(achieved_tf, 2), "peak": round(peak_tf, 2), "unit": "TFLOP/s",
                "frac": round(achieved_tf / peak_tf, 4),
                "traffic": traffic.get("bytes_per_launch") if traffic else None,
                "peak_source": "measured FFMA probe (tdc_probe_fma) on this GPU, this run",
                "flop_per_corr": FLOP_PER_CORR, "fp64_tflops_measured": round(fp64_tf, 3),
                "kernel": "focus_fp32_kernel"}

    out = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded point targets + complex Gaussian noise, FP64 jittered trajectory)",
           "config": bench_config(args, sc),
           "run": {"correlations_per_step": corr, "path": path, "anchor_pixels": p.lastStats()["anchor_pixels"]},
           "latency_ms": {"p50": round(float(np.percentile(step_ms, 50)), 3),
                          "p99": round(float(np.percentile(step_ms, 99)), 3)},
           "gpu_launches": 2 * args.steps, "clocks": clk, "roofline": roofline}

    if args.no_accuracy:
        print(json.dumps(out), flush=True)
        return
    # accuracy vs the FP64 oracle on a pixel sample (targets + random)
    import oracle

    build_oracle()
    pix = sample_pixels(sc, 1024)
    t = time.time()
    ref = oracle.focus(oracle_problem(sc, api, f64), oracle_opts(), pixels=pix)
    got = image[pix]
    sel = np.abs(ref) >= np.abs(ref).max() * 1e-2
    acc = {"rel_l2": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
           "max_phase_rad": float(np.max(np.abs(np.angle(got[sel] * np.conj(ref[sel]))))),
           "peak_err": float(abs(np.abs(got).max() - np.abs(ref).max()) / np.abs(ref).max()),
           "pixels": int(pix.size), "oracle": "FP64 on the same inputs"}
    out["accuracy"] = acc
    log(f"accuracy {acc} ({time.time() - t:.1f}s)")

    if not args.quick:
        # plain all-FP64-phase comparator on a row band of the same grid
        rows = max(8, min(args.side, 64))
        q = _sarlabtdc.TdcProcessor(0)
        band = np.ascontiguousarray(sc.grid[:rows])
        load(q, band)
        q.setPrecision("fp64")
        q.prepare(*start_args)
        q.uploadGrid()
        pimg = torch.empty(q.numPixels(), dtype=torch.complex64, device="cuda")
        q.focusDevice(pimg, stream)
        q.check(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q.focusDevice(pimg, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        q.check(stream)
        plain_gcorr = band.shape[0] * band.shape[1] * Cn * S / (e0.elapsed_time(e1) / 1e3) / 1e9
        pim = pimg.cpu().numpy()
        band_pix = pix[pix < pim.size]
        plain_acc = None
        if band_pix.size:
            rb = oracle.focus(oracle_problem(sc, api, f64), oracle_opts(), pixels=band_pix)
            plain_acc = float(np.linalg.norm(pim[band_pix] - rb) / np.linalg.norm(rb))
        out["plain"] = {"value": round(plain_gcorr, 2), "unit": UNIT, "speedup": round(kernel_gcorr / plain_gcorr, 2),
                        "rows": rows, "rel_l2": plain_acc, "kernel": "focus_fp64_kernel"}
        log(f"plain {out['plain']}")
        del q

        # FP32 general kernel: the same band with per-sample FP32 positions (the antenna keeps
        # moving during each chirp, ~0.3 mm per chirp), against the FP64 general kernel
        out["general"] = run_general(sc, api, band, rows, pix, stream, kernel_gcorr)
        log(f"general {out['general']}")

        # windowed focus of the whole grid: the antenna moving along the rail under a finite
        # Doppler band (zero-window chirps skipped, block tiles)
        out["windowed"] = run_windowed(sc, api, f64, stream, total_ms / args.steps)
        log(f"windowed {out['windowed']}")

        # e2e through the processor C ABI with host buffers
        e2e_steps = max(2, min(args.steps, 3))
        times, stats = [], None
        for i in range(1 + e2e_steps):
            t = time.perf_counter()
            load(p, sc.grid)
            p.start(*start_args)
            host_img = p.getFocusedImage()
            dt = time.perf_counter() - t
            stats = p.lastStats()
            if i > 0:
                times.append(dt)
        e2e_val = corr / float(np.mean(times)) / 1e9
        out["e2e"] = {"value": round(e2e_val, 2), "unit": UNIT, "h2d_bytes_per_step": int(stats["h2d_bytes"]),
                      "d2h_bytes_per_step": int(stats["d2h_bytes"]), "steps": e2e_steps,
                      "ms_per_step": round(1e3 * float(np.mean(times)), 2),
                      "stages_ms": {k: round(stats[k], 3) for k in ("h2d_ms", "prep_ms", "focus_ms", "d2h_ms",
                                                                      "total_ms")},
                      "kernel_launches_per_step": stats["kernel_launches"]}
        assert np.array_equal(host_img.ravel(), image), "e2e image differs from the device-resident image"
        log(f"e2e {out['e2e']}")

        cpu_g, npx, dt = time_oracle(sc, api, args.cpu_seconds, os.cpu_count(), f64)
        out["cpu_baseline"] = {"value": round(cpu_g, 4), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                               "sample": f"{npx} random pixels x {Cn} chirps x {S} samples ({dt:.1f}s), "
                                         "FP64 OpenMP oracle loop"}
        log(f"cpu {out['cpu_baseline']}")
        del p
        torch.cuda.empty_cache()
        if not args.no_serving:
            out["serving"] = serving_leg(args)
        if not args.no_autofocus:
            out["autofocus"] = autofocus_leg(args)
    print(json.dumps(out), flush=True)


def run_windowed(sc, api, f64, stream, unbounded_ms, speed=0.05, band_hz=10.0, n_check=192):
    """The same acquisition with the antenna moving at `speed` m/s along the rail and a
    `band_hz` Doppler band (tapered, fixed centre 0): device-resident focus time of the whole
    grid (median of 3 after a warm-up) and accuracy against the oracle on a pixel sample."""
    import torch

    import _sarlabtdc
    import oracle

    Cn, S = sc.n_pri, sc.n_samples
    vel = np.zeros((Cn, S, 3), np.float32)
    vel[..., 0] = speed
    q = _sarlabtdc.TdcProcessor(0)
    q.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], vel, api["attitude"],
                 api["modRate"], api["startFreq"], api["bodyBoresight"])
    if f64:
        q.setChirpPositionsF64(sc.positions)
        q.setFocusGridF64(sc.grid)
    else:
        q.setFocusGrid(np.ascontiguousarray(sc.grid, dtype=np.float32))
    q.prepare(0.0, band_hz, False, False, True)
    q.uploadGrid()
    img = torch.empty(q.numPixels(), dtype=torch.complex64, device="cuda")
    q.focusDevice(img, stream)
    q.check(stream)
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q.focusDevice(img, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    q.check(stream)
    stats = q.lastStats()
    ms = float(np.median(times))
    got = img.cpu().numpy()
    pix = sample_pixels(sc, n_check, seed=3)
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"],
                          position=sc.positions if f64 else api["position"][:, 0, :], velocity=vel,
                          modRate=api["modRate"], startFreq=api["startFreq"],
                          grid=sc.grid if f64 else sc.grid.astype(np.float32))
    ref = oracle.focus(prob, oracle.Opts(dopplerWinCenter=0.0, dopplerBandwidth=band_hz, applyRangeWin=False,
                                         dopplerWinTaper=True), pixels=pix)
    return {"ms": round(ms, 2), "unbounded_ms": round(unbounded_ms, 2),
            "speedup_vs_unbounded": round(unbounded_ms / ms, 2),
            "band_hz": band_hz, "speed_m_s": speed, "tile_cols": stats["tile_cols"],
            "span_permille": stats["span_permille"],
            "rel_l2": float(np.linalg.norm(got[pix] - ref) / np.linalg.norm(ref)), "pixels_checked": int(pix.size),
            "kernel": "focus_fp32_kernel<SKIP_ZERO>"}


def run_general(sc, api, band, rows, pix, stream, bulk_gcorr):
    """Per-sample trajectory on a row band: the default path for it (the smooth-motion kernel:
    the positions drift linearly within each chirp), the FP32 general kernel (smooth-motion
    path switched off) and the FP64 general kernel, each against the oracle on the band's
    sampled pixels."""
    import torch

    import _sarlabtdc
    import oracle

    Cn, S = sc.n_pri, sc.n_samples
    rng = np.random.default_rng(77)
    pos = np.broadcast_to(sc.positions[:, None, :], (Cn, S, 3)) + \
        (np.arange(S) / S)[None, :, None] * rng.normal(0.0, 0.3e-3, (Cn, 1, 3))
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    res = {}
    band_pix = pix[pix < band.shape[0] * band.shape[1]]
    ref = None
    for name, precision, motion, n_rows in (("fp32", "fp32", True, rows), ("fp32_general", "fp32", False, rows),
                                            ("fp64", "fp64", True, max(2, rows // 8))):
        q = _sarlabtdc.TdcProcessor(0)
        q.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], pos, api["velocity"], api["attitude"],
                     api["modRate"], api["startFreq"], api["bodyBoresight"])
        g = np.ascontiguousarray(band[:n_rows], dtype=np.float32)
        q.setFocusGrid(g)
        q.setPrecision(precision)
        q.setMotionPath(motion)
        q.prepare(0.0, float("inf"), False, False, True)
        q.uploadGrid()
        gimg = torch.empty(q.numPixels(), dtype=torch.complex64, device="cuda")
        q.focusDevice(gimg, stream)
        q.check(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        q.focusDevice(gimg, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        q.check(stream)
        gcorr = g.shape[0] * g.shape[1] * Cn * S / (e0.elapsed_time(e1) / 1e3) / 1e9
        gim = gimg.cpu().numpy()
        sel = band_pix[band_pix < gim.size]
        acc = None
        if sel.size:
            prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=pos,
                                  modRate=api["modRate"], startFreq=api["startFreq"], grid=g)
            r = oracle.focus(prob, oracle_opts(), pixels=sel)
            acc = float(np.linalg.norm(gim[sel] - r) / np.linalg.norm(r))
        res[name] = {"value": round(gcorr, 2), "rows": n_rows, "path": q.path(), "rel_l2": acc,
                     "motion_segment": q.lastStats()["motion_segment"]}
        del q
    kernels = {"fp32_motion": "focus_motion_kernel", "general": "focus_general_kernel"}
    return {"value": res["fp32"]["value"], "unit": UNIT, "kernel": kernels.get(res["fp32"]["path"], res["fp32"]["path"]),
            "workload": "per-sample FP32 positions drifting ~0.3 mm within each chirp, same band",
            "fp32": res["fp32"], "fp32_general": res["fp32_general"], "fp64": res["fp64"],
            "speedup_vs_general": round(res["fp32"]["value"] / res["fp32_general"]["value"], 2),
            "speedup_vs_fp64": round(res["fp32"]["value"] / res["fp64"]["value"], 2),
            "vs_bulk": round(res["fp32"]["value"] / bulk_gcorr, 4)}


def run_general_only(args):
    """The general-kernel leg of the precision-study scene on its own (a JSON line)."""
    import torch

    assert torch.cuda.is_available(), "bench.py needs a CUDA device"
    torch.cuda.set_device(0)
    sc = make_scene(args, "cuda")
    api = sc.api_arrays()
    rows = max(8, min(args.side, 64))
    band = np.ascontiguousarray(sc.grid[:rows])
    pix = sample_pixels(sc, 192)
    build_oracle()
    res = run_general(sc, api, band, rows, pix, torch.cuda.current_stream(), float("nan"))
    res.pop("vs_bulk", None)
    out = {"metric": "FP32 general kernel: Gcorr/s on per-sample trajectories", "unit": UNIT,
           "value": res["value"], "higher_is_better": True, "dtype": "f32", "n_gpus": 1,
           "config": {"workload": f"{rows} x {args.side} px band of the precision study, {sc.n_pri} chirps x "
                                  f"{sc.n_samples} samples, FP32 positions drifting ~0.3 mm within each chirp"},
           "general": res}
    print(json.dumps(out), flush=True)


def serving_leg(args):
    """Config 4: a seeded Poisson stream of focus requests through the request loop, against
    the same jobs run one after another through the processor (FIFO, same arrival times).
    Returns the `serving` object (with the clocks sampled while both ran)."""
    import threading

    from sarlabtdc import scenes
    from sarlabtdc.serving import FocusServer

    rng = np.random.default_rng(4)
    n = args.jobs
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n))
    sides = rng.choice([128, 256, 512, 1024, 2048], n)
    chirps = np.round(np.exp(rng.uniform(np.log(256), np.log(8192), n))).astype(int)
    samples = rng.choice([256, 512, 1024], n)
    ntg = rng.integers(1, 101, n)
    t = time.time()
    jobs = []
    for i in range(n):
        radar = scenes.Radar(n_samples=int(samples[i]))
        pos = scenes.rail(int(chirps[i]), int(chirps[i]) * 0.25e-3, 0.3)
        side = int(sides[i])
        grid = scenes.ground_grid(side, side, 1.0 / side, y0=0.3).astype(np.float32)
        lo, hi = grid.reshape(-1, 3).min(0), grid.reshape(-1, 3).max(0)
        tg = np.zeros((int(ntg[i]), 3))
        tg[:, 0] = rng.uniform(lo[0], hi[0], tg.shape[0])
        tg[:, 1] = rng.uniform(lo[1], hi[1], tg.shape[0])
        amps = np.exp(2j * np.pi * rng.uniform(0, 1, tg.shape[0]))
        raw = scenes.simulate_raw(pos, tg, amps, radar, "cuda").astype(np.complex64)
        jobs.append(dict(raw=raw, st=radar.sample_times(), pos=pos.astype(np.float32), grid=grid,
                         K=np.float32(radar.mod_rate), f0=np.float32(radar.f0),
                         corr=side * side * int(chirps[i]) * int(samples[i])))
    log(f"serving: generated {n} jobs in {time.time() - t:.0f}s; "
        f"{sum(j['corr'] for j in jobs) / 1e12:.1f} Tcorr total")
    start = (0.0, float("inf"), False, False, True)

    clocks = Clocks()
    clocks.start()
    # request loop
    with FocusServer(max_jobs=16) as srv:
        ids = [None] * n
        t0 = time.perf_counter()

        def client():
            for i, j in enumerate(jobs):
                dt = arrivals[i] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                ids[i] = srv.submit(j["raw"], j["st"], j["pos"], j["grid"], j["K"], j["f0"], start=start)

        th = threading.Thread(target=client)
        th.start()
        th.join()
        infos = [srv.wait(i)[1] for i in ids]
        st = srv.stats()
    lat = np.array([x["done_ms"] - x["submit_ms"] for x in infos])
    span = max(x["done_ms"] for x in infos) - min(x["submit_ms"] for x in infos)
    total = sum(j["corr"] for j in jobs)
    served = {"p50_ms": round(float(np.percentile(lat, 50)), 1), "p99_ms": round(float(np.percentile(lat, 99)), 1),
              "gcorr_s": round(total / (span / 1e3) / 1e9, 1), "span_s": round(span / 1e3, 2),
              "launches": st["launches"]}
    log(f"request loop: {served}")

    # serial: the same jobs one after another through the processor (tdc_processor_start: each
    # job's whole focus in one launch, its image copied out), FIFO on the same arrivals
    import ctypes

    import _sarlabtdc
    import _tdc_capi as L

    lib = L.lib()
    proc = _sarlabtdc.TdcProcessor(0)
    bore = np.array([0.0, 1.0, 0.0], np.float32)
    service = []
    for j in jobs:
        t = time.perf_counter()
        n_pri, n_s = j["raw"].shape
        rows, cols = j["grid"].shape[:2]
        # per-chirp positions: the per-sample arrays of setRawData are replaced by the trajectory
        L.check(lib.tdc_processor_set_raw_data(proc._h, L.ptr(j["raw"]), None, L.ptr(j["st"]), L.ptr(j["pos"]), None,
                                               None, n_pri, n_s, float(j["K"]), float(j["f0"]), L.ptr(bore)))
        L.check(lib.tdc_processor_set_trajectory_per_chirp(proc._h, L.ptr(j["pos"]), None, None))
        L.check(lib.tdc_processor_set_focus_grid(proc._h, L.ptr(j["grid"]), rows, cols))
        L.check(lib.tdc_processor_start(proc._h, *start[:2], int(start[2]), int(start[3]), int(start[4])))
        buf = lib.tdc_processor_image_buffer(proc._h)
        img = np.empty(rows * cols, np.complex64)
        ctypes.memmove(img.ctypes.data, buf, img.nbytes)
        service.append(time.perf_counter() - t)
    del proc
    finish, lat_s = 0.0, []
    for a, sv in zip(arrivals, service):
        finish = max(finish, a) + sv
        lat_s.append(finish - a)
    lat_s = np.array(lat_s) * 1e3
    clk = clocks.stop()
    serial = {"p50_ms": round(float(np.percentile(lat_s, 50)), 1), "p99_ms": round(float(np.percentile(lat_s, 99)), 1),
              "gcorr_s": round(total / (finish - arrivals[0]) / 1e9, 1), "span_s": round(finish - arrivals[0], 2)}
    log(f"serial: {serial}")
    return {"workload": f"serving mix: {n} requests, Poisson {args.rate}/s, grids 128^2..2048^2, "
                        "256..8192 chirps (log-uniform), 256/512/1024 samples, 1-100 targets",
            "unit": UNIT, "total_correlations": total, "request_loop": served, "serial_processor": serial,
            "offered_gcorr_s": round(total / (arrivals[-1] - arrivals[0]) / 1e9, 1),
            "serial_how": "the same jobs one after another through the processor (tdc_processor_start, each "
                          "job's focus in one launch), FIFO on the same arrivals (latency = queueing on those "
                          "arrivals + measured service time)",
            "clocks": clk}


def run_windowed_only(args):
    """The windowed leg of the precision-study scene on its own (a JSON line): the whole grid
    with the antenna moving along the rail under a 10 Hz Doppler band."""
    import torch

    assert torch.cuda.is_available(), "bench.py needs a CUDA device"
    torch.cuda.set_device(0)
    sc = make_scene(args, "cuda")
    build_oracle()
    res = run_windowed(sc, sc.api_arrays(), True, torch.cuda.current_stream(), float("nan"))
    res.pop("unbounded_ms", None)
    res.pop("speedup_vs_unbounded", None)
    out = {"metric": "windowed focus: ms per focus", "unit": "ms", "value": res["ms"], "higher_is_better": False,
           "dtype": "f32", "n_gpus": 1,
           "config": {"workload": f"{args.side}x{args.side} px precision-study grid, {sc.n_pri} chirps x "
                                  f"{sc.n_samples} samples, antenna at 0.05 m/s along the rail, 10 Hz band"},
           "windowed": res}
    print(json.dumps(out), flush=True)


def run_serving(args):
    """Config 4 alone: one JSON line."""
    sv = serving_leg(args)
    served = sv["request_loop"]
    out = {"metric": "serving: p50/p99 focus latency and aggregate Gcorr/s", "value": served["gcorr_s"],
           "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded Poisson arrivals, point targets)",
           "config": {"workload": sv["workload"], "total_correlations": sv["total_correlations"]},
           "latency_ms": {"p50": served["p50_ms"], "p99": served["p99_ms"]},
           "request_loop": served, "serial_processor": sv["serial_processor"],
           "offered_gcorr_s": sv["offered_gcorr_s"], "clocks": sv["clocks"]}
    print(json.dumps(out), flush=True)


def autofocus_leg(args):
    """Config 5: entropy autofocus of a random-walk trajectory error through the adjoint kernel.
    Returns the `autofocus` object (with the clocks sampled while it ran)."""
    import torch

    import _sarlabtdc
    import oracle
    from sarlabtdc import autofocus, scenes

    sc = scenes.autofocus_scene(device="cuda")
    api = sc.api_arrays()
    p = _sarlabtdc.TdcProcessor(0)
    p.setRawData(*api.values())
    p.setChirpPositionsF64(sc.positions)
    p.setFocusGridF64(sc.grid)
    op = autofocus.FocusOperator(p, (0.0, float("inf"), False, False, True))
    corr = sc.correlations()
    clocks = Clocks()
    clocks.start()
    # timing of forward and adjoint
    zero = torch.zeros((sc.n_pri, 3), dtype=torch.float64, device="cuda")
    g = torch.randn(op.n_pix, dtype=torch.complex64, device="cuda")
    op.image(zero)
    op.adjoint(zero, g)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd_runs, adj_runs = [], []
    for _ in range(5):
        e[0].record()
        img = op.image(zero)
        e[1].record()
        op.adjoint(zero, g)
        e[2].record()
        torch.cuda.synchronize()
        fwd_runs.append(e[0].elapsed_time(e[1]))
        adj_runs.append(e[1].elapsed_time(e[2]))
    fwd_ms, adj_ms = float(np.median(fwd_runs)), float(np.median(adj_runs))
    adj_kept = bool(p.lastStats()["adjoint_stored"])
    # the same adjoint recomputing the forward's sums instead of reading them
    p.keepChirpSums(False)
    op.adjoint(zero, g)
    torch.cuda.synchronize()
    e[1].record()
    op.adjoint(zero, g)
    e[2].record()
    torch.cuda.synchronize()
    adj_full_ms = e[1].elapsed_time(e[2])
    p.keepChirpSums(True)
    # gradient check on a pixel subset: engine adjoint vs FP64 oracle and vs FD of the engine
    rng = np.random.default_rng(55)
    pix = rng.choice(op.n_pix, 96, replace=False)
    gsub = np.zeros(op.n_pix, np.complex64)
    gsub[pix] = (rng.normal(size=pix.size) + 1j * rng.normal(size=pix.size)).astype(np.complex64)
    off = rng.normal(0, 0.05e-3, (sc.n_pri, 3))
    got = op.adjoint(torch.from_numpy(off).cuda(), torch.from_numpy(gsub).cuda()).cpu().numpy()
    build_oracle()
    prob = oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions,
                          modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid)
    ref = oracle.adjoint_offsets(prob, oracle_opts(), off, gsub[pix].astype(np.complex128), pixels=pix)
    grad_err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    h = 1e-6
    fd_rel = []
    offt = torch.from_numpy(off).cuda()
    for c, k in [(100, 0), (2000, 1), (3500, 2)]:
        ep = np.array(off)
        em = np.array(off)
        ep[c, k] += h
        em[c, k] -= h
        lp = float(np.real(np.sum(np.conj(gsub[pix]) * oracle.focus(
            oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions + ep,
                           modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid), oracle_opts(),
            pixels=pix))))
        lm = float(np.real(np.sum(np.conj(gsub[pix]) * oracle.focus(
            oracle.Problem(raw=api["rawData"], sampleTimes=api["sampleTimes"], position=sc.positions + em,
                           modRate=api["modRate"], startFreq=api["startFreq"], grid=sc.grid), oracle_opts(),
            pixels=pix))))
        fd = (lp - lm) / (2 * h)
        fd_rel.append(abs(got[c, k] - fd) / max(abs(fd), 1e-30))
    # autofocus
    walk = sc.meta["walk"]
    centre = sc.grid.reshape(-1, 3).mean(0)
    lam = float(oracle.wavelength_center(api["sampleTimes"], api["modRate"], api["startFreq"]))
    ph0 = autofocus.residual_phase_rms(np.zeros_like(walk), walk, sc.positions, centre, lam)
    ideal = op.image(torch.from_numpy(walk).cuda()).cpu().numpy()
    coh0 = autofocus.coherence(op.image(None).cpu().numpy(), ideal)
    res = autofocus.autofocus(op, steps=args.af_steps, lr=args.af_lr)
    ph1 = autofocus.residual_phase_rms(res.offsets.cpu().numpy(), walk, sc.positions, centre, lam)
    coh1 = autofocus.coherence(op.image(res.offsets).cpu().numpy(), ideal)
    # warm start: a smooth estimate of the trajectory error (the walk averaged by a 64-point
    # piecewise-linear fit, ~32 mm of rail per segment), refined over a 256-point basis
    B64 = autofocus.hat_basis(sc.n_pri, 64, "cpu").numpy()
    prior = B64 @ np.linalg.lstsq(B64, walk, rcond=None)[0]
    prior_t = torch.from_numpy(prior).cuda()
    ph_w0 = autofocus.residual_phase_rms(prior, walk, sc.positions, centre, lam)
    coh_w0 = autofocus.coherence(op.image(prior_t).cpu().numpy(), ideal)
    warm = autofocus.autofocus(op, steps=args.af_steps, lr=2e-4, offsets=prior_t, knots=256)
    ph_w1 = autofocus.residual_phase_rms(warm.offsets.cpu().numpy(), walk, sc.positions, centre, lam)
    coh_w1 = autofocus.coherence(op.image(warm.offsets).cpu().numpy(), ideal)
    clk = clocks.stop()
    out = {"workload": "autofocus: 512x512 px @1mm, 4096 chirps x 1024 samples over 2 m, random walk 0.2 mm/step",
           "correlations_per_forward": corr,
           # (the first step also allocates the kept per-chirp sums, C x P x 8 bytes: reported apart)
           "step_ms": {"p50": round(float(np.median(res.step_ms)), 2), "mean": round(float(np.mean(res.step_ms[1:])), 2),
                       "max": round(float(np.max(res.step_ms[1:])), 2), "first": round(float(res.step_ms[0]), 2)},
           "forward_ms": round(fwd_ms, 2), "adjoint_ms": round(adj_ms, 2), "adjoint_read_kept_sums": adj_kept,
           "adjoint_recomputing_ms": round(adj_full_ms, 2),
           "forward_gcorr_s": round(corr / (fwd_ms / 1e3) / 1e9, 1),
           "adjoint_gcorr_s": round(corr / (adj_ms / 1e3) / 1e9, 1),
           "gradient_vs_fp64_oracle_rel_l2": grad_err, "gradient_pixels": int(pix.size),
           "gradient_vs_central_fd_h1e-6_rel": fd_rel,
           "entropy": {"start": res.entropy[0], "end": res.entropy[-1]},
           "residual_phase_rms_rad": {"start": ph0, "end": ph1},
           "coherence_with_true_trajectory_image": {"start": coh0, "end": coh1},
           "adam_steps": args.af_steps, "lr_m": args.af_lr,
           "warm_start": {"start": "the true walk averaged by a 64-point piecewise-linear fit (a smooth "
                                   "trajectory estimate)", "knots": 256, "adam_steps": args.af_steps, "lr_m": 2e-4,
                          "entropy": {"start": warm.entropy[0], "end": warm.entropy[-1]},
                          "residual_phase_rms_rad": {"start": ph_w0, "end": ph_w1},
                          "coherence_with_true_trajectory_image": {"start": coh_w0, "end": coh_w1}},
           "clocks": clk}
    del op, p
    torch.cuda.empty_cache()
    return out


def run_autofocus(args):
    """Config 5 alone: one JSON line."""
    af = autofocus_leg(args)
    out = {"metric": "autofocus: adjoint accuracy, entropy, residual phase, time per Adam step",
           "value": af["step_ms"]["p50"], "unit": "ms/Adam step (median)", "higher_is_better": False,
           "n_gpus": 1, "dtype": "f32", "data": "synthetic (seeded random-walk trajectory error, 30 targets)",
           "config": {"workload": af["workload"], "correlations_per_forward": af["correlations_per_forward"]},
           **{k: v for k, v in af.items() if k not in ("workload", "correlations_per_forward")}}
    print(json.dumps(out), flush=True)


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import torch

    build_oracle()
    device = "cuda" if torch.cuda.is_available() else "cpu"
    sc = make_scene(args, device)
    api = sc.api_arrays()
    cores = os.cpu_count()
    import oracle

    prob = oracle_problem(sc, api, uses_f64(args))
    o = oracle_opts()
    rng = np.random.default_rng(99)
    per_px = sc.n_pri * sc.n_samples
    # size one step to ~budget seconds of CPU work
    t = time.perf_counter()
    oracle.focus(prob, o, pixels=rng.choice(sc.n_pix, 8, replace=False), threads=cores)
    dt = time.perf_counter() - t
    budget = max(2.0, min(15.0, 100.0 / max(1, args.steps + args.warmup)))
    npx = int(max(8, min(sc.n_pix, 8 * budget / max(dt, 1e-3))))
    for _ in range(args.warmup):
        oracle.focus(prob, o, pixels=rng.choice(sc.n_pix, max(8, npx // 8), replace=False), threads=cores)
    times = []
    for _ in range(args.steps):
        pix = rng.choice(sc.n_pix, npx, replace=False)
        t = time.perf_counter()
        oracle.focus(prob, o, pixels=pix, threads=cores)
        times.append(time.perf_counter() - t)
    value = npx * per_px / float(np.mean(times)) / 1e9
    out = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * float(np.mean(times)), 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": "synthetic (seeded point targets + complex Gaussian noise, FP64 jittered trajectory)",
           "config": bench_config(args, sc),
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"{npx} random pixels per step x {sc.n_pri} chirps x {sc.n_samples} samples; "
                                      "the reference has no CPU focus path: FP64 OpenMP restatement of "
                                      "tdckernels.cu:70-315 (oracle/)"},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_sharded(args):
    """N GPUs, one process each (torchrun): pixel sharding with weak scaling. Every rank holds
    the whole precision-study acquisition and focuses its own 1024-row block of a grid of
    N x 1024 rows (the scene's grid shifted by its block along y), planned for the whole grid
    (setPlanPixels). No data moves between ranks while they focus; `value` = all ranks'
    correlations / the slowest rank's time. `e2e`: the sharded processor with host buffers
    (setRawData, setFocusGrid, start, the image gathered on every rank)."""
    import torch
    import torch.distributed as dist

    import _sarlabtdc
    from sarlabtdc import sharding

    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    sc = make_scene(args, "cuda")
    api = sc.api_arrays()
    rows, cols = sc.grid.shape[:2]
    grid = sc.grid.copy()
    grid[..., 1] += rank * rows * 1e-3
    corr = sc.correlations()
    start_args = (0.0, float("inf"), False, False, True)
    p = _sarlabtdc.TdcProcessor(local)
    p.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                 api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
    p.setChirpPositionsF64(sc.positions)
    p.setFocusGridF64(grid)
    p.setPlanPixels(world * rows * cols)
    p.prepare(*start_args)
    p.uploadGrid()
    img = torch.empty(sc.n_pix, dtype=torch.complex64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(max(3, args.warmup)):
        p.focusDevice(img, stream)
        flush.zero_()
    p.check(stream)
    clocks = Clocks()
    if rank == 0:
        clocks.start()
        time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for e0, e1 in evs:
        e0.record(stream)
        p.focusDevice(img, stream)
        e1.record(stream)
        flush.zero_()
    torch.cuda.synchronize()
    wall = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
    dist.barrier()
    clk = clocks.stop() if rank == 0 else None
    p.check(stream)
    kernel_ms = torch.tensor([float(np.mean([a.elapsed_time(b) for a, b in evs]))], dtype=torch.float64,
                             device="cuda")
    dist.all_reduce(wall, op=dist.ReduceOp.MAX)
    dist.all_reduce(kernel_ms, op=dist.ReduceOp.MAX)
    total_s = float(wall.item())
    value = world * corr * args.steps / total_s / 1e9

    # e2e: host buffers through the sharded processor, image gathered on every rank
    tall = np.concatenate([sc.grid + np.array([0.0, r * rows * 1e-3, 0.0]) for r in range(world)], axis=0)
    sp = sharding.ShardedProcessor(local, rank, world)
    times = []
    for i in range(3):
        dist.barrier()
        t = time.perf_counter()
        sp.setRawData(api["rawData"], api["priTimes"], api["sampleTimes"], api["position"], api["velocity"],
                      api["attitude"], api["modRate"], api["startFreq"], api["bodyBoresight"])
        sp.setChirpPositionsF64(sc.positions)
        sp.setFocusGridF64(tall)
        sp.start(*start_args)
        full = sp.getFocusedImage()
        dt = torch.tensor([time.perf_counter() - t], dtype=torch.float64, device="cuda")
        dist.all_reduce(dt, op=dist.ReduceOp.MAX)
        if i > 0:
            times.append(float(dt.item()))
    stats = sp.proc.lastStats()
    if rank == 0:
        peak_tf, fp64_tf, _ = fp32_peak_tflops(_tdc_lib(), torch)
        achieved = corr / (float(kernel_ms.item()) / 1e3) / 1e9 * FLOP_PER_CORR / 1e3
        out = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": round(1e3 * total_s / args.steps, 3), "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded point targets + complex Gaussian noise, FP64 jittered trajectory)",
               "config": bench_config(args, sc),
               "run": {"correlations_per_step": world * corr, "sharding": f"{world} row blocks of {rows} x {cols} "
                       "pixels, one per GPU, the whole acquisition on every GPU, no collective while focusing",
                       "path": p.path()},
               "gpu_launches": 2 * args.steps, "clocks": clk,
               "roofline": {"bound": "fp32", "achieved": round(achieved, 2), "peak": round(peak_tf, 2),
                            "unit": "TFLOP/s", "frac": round(achieved / peak_tf, 4), "traffic": None,
                            "peak_source": "measured FFMA probe (tdc_probe_fma) on rank 0's GPU, this run",
                            "kernel": "focus_fp32_kernel (slowest rank)"},
               "e2e": {"value": round(world * corr / float(np.mean(times)) / 1e9, 2), "unit": UNIT,
                       "h2d_bytes_per_step": int(stats["h2d_bytes"]) * world,
                       "d2h_bytes_per_step": int(stats["d2h_bytes"]) * world, "steps": len(times),
                       "gathered_image_bytes": int(full.nbytes)}}
        print(json.dumps(out), flush=True)
    dist.barrier()
    dist.destroy_process_group()


def _tdc_lib():
    import _tdc_capi

    return _tdc_capi.lib()


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "ours" and (args.gpus > 1 or world > 1):
        if world != args.gpus or args.config != "2":
            print(json.dumps({"error": "--gpus N runs the precision study under torchrun with N processes"}))
            return 2
        run_sharded(args)
        return 0
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "4":
        run_serving(args)
    elif args.config == "5":
        run_autofocus(args)
    elif args.general_only:
        run_general_only(args)
    elif args.windowed_only:
        run_windowed_only(args)
    else:
        run_ours(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
