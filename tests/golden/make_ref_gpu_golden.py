"""Golden focused images from the reference's own GPU kernels.

Runs on a machine with a GPU and oracle/_ref/tdckernels.ptx, which
oracle/build.py compiles from the reference's tdc-lib/src/tdckernels.cu where
it lies in the reference checkout:

    python oracle/build.py                       # next to the reference checkout
    python tests/golden/make_ref_gpu_golden.py   # on the GPU machine

The reference kernels (initRangeWindowKernel, createWindowKernel,
referenceResponseKernel, correlateWithReference) are loaded from the PTX with
the CUDA driver API and launched in the order and with the launch shapes of the
reference's host code (tdc-lib/src/tdcprocessor.cpp:59-167, tdckernels.cu
wrappers): per chunk of 128 PRIs the valid rows are staged (rows past them keep
the previous chunk's values) and copied whole; per pixel the host skip test,
then window, reference response and correlation kernels; the chunk's sum
(nppsSum_32fc in the reference) is taken in FP64, rounded to complex float and
added to the float pixel (addToImage). The inputs and the resulting images are
written to tests/golden/ref_gpu_images.npz.
"""
from __future__ import annotations

import ctypes as C
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "sarlab-tdc_gb300"))

CHUNK = 128
OUT = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent / "ref_gpu_images.npz"

# Itanium-mangled names of the reference kernels (tdckernels.cu:32, :70, :178, :250).
K_RANGE = b"_Z21initRangeWindowKernelPfib"
K_WINDOW = b"_Z18createWindowKernelPfPKfPK6float3S4_PK6float4S2_S2_fffbbiii"
K_REF = b"_Z23referenceResponseKernelP6float2PKfPK6float3S2_S3_ffiii"
K_CORR = b"_Z22correlateWithReferencePK6float2PS_iii"


class F3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Driver:
    def __init__(self, ptx: bytes):
        import torch

        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self._ck(self.cu.cuModuleLoadData(C.byref(self.mod), C.c_char_p(ptx + b"\0")), "cuModuleLoadData")
        self.fn = {}
        for name in (K_RANGE, K_WINDOW, K_REF, K_CORR):
            f = C.c_void_p()
            self._ck(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name), name.decode())
            self.fn[name] = f

    @staticmethod
    def _ck(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def launch(self, name, grid, block, args):
        objs = []
        for a in args:
            objs.append(a)
        ptrs = (C.c_void_p * len(objs))(*[C.cast(C.pointer(o), C.c_void_p) for o in objs])
        self._ck(self.cu.cuLaunchKernel(self.fn[name], grid[0], grid[1], 1, block[0], block[1], 1, 0, None, ptrs,
                                        None), name.decode())


def ptr(t):
    return C.c_uint64(t.data_ptr())


def skip_nonzero(pos_st, vel_st, att_st, S, tgt, bore, lam, center, bw, centroid):
    """tdcprocessor.cpp:347-383 on the staging arrays (FP64 arithmetic)."""
    import oracle
    from oracle import oracle as O

    rows, samples = oracle.skip_points(S, CHUNK)
    vals = []
    for r in rows:
        for s in samples:
            p, v, q = pos_st[r, s].astype(np.float64), vel_st[r, s].astype(np.float64), att_st[r, s].astype(np.float64)
            if centroid:
                ant = np.zeros(3)
                O.lib().tdco_q_rot(O._ptr(np.ascontiguousarray(q), O.C.c_double),
                                   O._ptr(np.ascontiguousarray(np.asarray(bore, np.float64)), O.C.c_double),
                                   O._ptr(ant, O.C.c_double))
                fc = 2.0 / lam * float(np.dot(v, ant))
            else:
                fc = float(np.float32(center))
            d = tgt - p
            n = np.linalg.norm(d)
            fd = 2.0 / lam * float(np.dot(v, d)) / n if n > 0 else float("nan")
            vals.append(abs(fd - fc))
    m = vals[0]
    for x in vals[1:]:
        if x < m:
            m = x
    return m <= float(np.float32(bw)) / 2.0


def per_sample(a, n_pri, n_samples):
    """[C, k] per-chirp rows broadcast to the reference's [C, S, k], or [C, S, k] as given."""
    a = np.asarray(a, np.float32)
    if a.ndim == 2:
        a = np.broadcast_to(a[:, None, :], (n_pri, n_samples, a.shape[1]))
    return np.ascontiguousarray(a)


def reference_focus(drv, case, host_skip=True, device_sum=False):
    """The reference's per-(chunk, pixel) launch sequence. host_skip=False leaves out the
    host skip test (it passes every chunk under an infinite band); device_sum=True keeps
    the chunk sums and the image on the device (FP64 sum rounded to complex float, then
    added, as nppsSum_32fc + addToImage do) instead of adding them on the host."""
    import torch

    import oracle

    raw, st = case["raw"], case["sample_times"]
    C_, S = raw.shape
    pos, vel, att = (per_sample(case[k], C_, S) for k in ("pos", "vel", "att"))
    grid = case["grid"].reshape(-1, 3).astype(np.float32)
    K, f0 = float(np.float32(case["mod_rate"])), float(np.float32(case["start_freq"]))
    center, bw = float(case["center"]), float(case["bw"])
    centroid, apply_rw, taper = bool(case["centroid"]), bool(case["apply_range_win"]), bool(case["taper"])
    bore = tuple(float(b) for b in case["bore"])
    lam = float(oracle.wavelength_center(st, K, f0))
    dev = "cuda"
    rw = torch.empty(S, dtype=torch.float32, device=dev)
    drv.launch(K_RANGE, ((S + 31) // 32, 1), (32, 1), [ptr(rw), C.c_int(S), C.c_bool(apply_rw)])
    st_d = torch.from_numpy(np.ascontiguousarray(st, np.float32)).to(dev)
    n = CHUNK * S
    raw_d = torch.zeros(n * 2, dtype=torch.float32, device=dev)
    pos_d = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    vel_d = torch.zeros(n * 3, dtype=torch.float32, device=dev)
    att_d = torch.zeros(n * 4, dtype=torch.float32, device=dev)
    win_d = torch.zeros(n, dtype=torch.float32, device=dev)
    ref_d = torch.zeros(n * 2, dtype=torch.float32, device=dev)
    raw_st = np.zeros((CHUNK, S), np.complex64)
    pos_st = np.zeros((CHUNK, S, 3), np.float32)
    vel_st = np.zeros((CHUNK, S, 3), np.float32)
    att_st = np.zeros((CHUNK, S, 4), np.float32)
    image = np.zeros(grid.shape[0], np.complex64)
    image_d = torch.zeros(grid.shape[0], dtype=torch.complex64, device=dev) if device_sum else None
    grid_blk = ((S + 15) // 16, CHUNK // 16)
    for k in range((C_ + CHUNK - 1) // CHUNK):
        valid = min(CHUNK, C_ - k * CHUNK)
        sl = slice(k * CHUNK, k * CHUNK + valid)
        raw_st[:valid], pos_st[:valid], vel_st[:valid], att_st[:valid] = raw[sl], pos[sl], vel[sl], att[sl]
        raw_d.copy_(torch.from_numpy(raw_st.view(np.float32).ravel()))
        pos_d.copy_(torch.from_numpy(pos_st.ravel()))
        vel_d.copy_(torch.from_numpy(vel_st.ravel()))
        att_d.copy_(torch.from_numpy(att_st.ravel()))
        for pix in range(grid.shape[0]):
            tgt = grid[pix]
            if host_skip and not skip_nonzero(pos_st, vel_st, att_st, S, tgt.astype(np.float64), bore, lam, center,
                                              bw, centroid):
                continue
            T = F3(*[float(x) for x in tgt])
            B = F3(*bore)
            drv.launch(K_WINDOW, grid_blk, (16, 16),
                       [ptr(win_d), ptr(rw), ptr(pos_d), ptr(vel_d), ptr(att_d), T, B, C.c_float(lam),
                        C.c_float(bw), C.c_float(center), C.c_bool(centroid), C.c_bool(taper), C.c_int(k),
                        C.c_int(C_), C.c_int(S)])
            drv.launch(K_REF, grid_blk, (16, 16),
                       [ptr(ref_d), ptr(win_d), ptr(pos_d), ptr(st_d), T, C.c_float(f0), C.c_float(K), C.c_int(k),
                        C.c_int(C_), C.c_int(S)])
            drv.launch(K_CORR, grid_blk, (16, 16), [ptr(raw_d), ptr(ref_d), C.c_int(k), C.c_int(C_), C.c_int(S)])
            if device_sum:
                v = ref_d[: 2 * valid * S].view(-1, 2).double().sum(0).float()
                image_d[pix] += torch.complex(v[0], v[1])
                continue
            v = ref_d[: 2 * valid * S].view(-1, 2).double().sum(0).cpu().numpy()
            image[pix] = np.complex64(image[pix] + np.complex64(complex(v[0], v[1])))
    torch.cuda.synchronize()
    return image_d.cpu().numpy() if device_sum else image


def make_cases():
    from sarlabtdc import scenes

    cases = {}
    # A: plain stripmap, reference Hamming range window, partial last chunk (200 = 128 + 72)
    sc = scenes.small_scene(seed=101, n_pri=200, n_samples=64, nx=12, ny=10, jitter=0.2e-3, device="cuda")
    cases["plain"] = dict(raw=sc.raw, sample_times=sc.radar.sample_times(), pos=sc.positions.astype(np.float32),
                          vel=np.zeros((200, 3), np.float32), att=np.tile([1, 0, 0, 0], (200, 1)).astype(np.float32),
                          grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                          start_freq=np.float32(sc.radar.f0), center=0.0, bw=float("inf"), centroid=0,
                          apply_range_win=1, taper=1, bore=np.array([0, 1, 0], np.float32))
    # B: moving antenna, centroid Doppler window with taper, skip test, 300 PRIs (stale rows)
    rng = np.random.default_rng(102)
    sc = scenes.small_scene(seed=103, n_pri=300, n_samples=48, nx=11, ny=9, rail_len=0.3, device="cuda")
    yaw = rng.normal(0, 0.02, 300)
    att = np.stack([np.cos(yaw / 2), 0 * yaw, 0 * yaw, np.sin(yaw / 2)], 1).astype(np.float32)
    vel = np.zeros((300, 3), np.float32)
    vel[:, 0] = 0.05
    cases["doppler"] = dict(raw=sc.raw, sample_times=sc.radar.sample_times(), pos=sc.positions.astype(np.float32),
                            vel=vel, att=att, grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                            start_freq=np.float32(sc.radar.f0), center=2.0, bw=18.0, centroid=1, apply_range_win=1,
                            taper=1, bore=np.array([0, 1, 0], np.float32))
    # C: rectangular window with a fixed centre, exactly two chunks, no range window
    sc = scenes.small_scene(seed=104, n_pri=256, n_samples=40, nx=10, ny=8, rail_len=0.4, device="cuda")
    vel = np.zeros((256, 3), np.float32)
    vel[:, 0] = 0.04
    cases["rect"] = dict(raw=sc.raw, sample_times=sc.radar.sample_times(), pos=sc.positions.astype(np.float32),
                         vel=vel, att=np.tile([1, 0, 0, 0], (256, 1)).astype(np.float32),
                         grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                         start_freq=np.float32(sc.radar.f0), center=1.0, bw=24.0, centroid=0, apply_range_win=0,
                         taper=0, bore=np.array([0, 1, 0], np.float32))
    # D: per-sample trajectory: the antenna keeps moving within each chirp (positions drift
    # up to ~0.5 mm per chirp), per-sample velocity, centroid window with taper, skip test,
    # 200 PRIs (a partial last chunk)
    rng = np.random.default_rng(105)
    sc = scenes.small_scene(seed=106, n_pri=200, n_samples=48, nx=10, ny=9, rail_len=0.3, device="cuda")
    C_, S = 200, 48
    frac = (np.arange(S) / S)[None, :, None]
    pos = sc.positions[:, None, :] + frac * rng.normal(0.0, 0.3e-3, (C_, 1, 3))
    vel = np.zeros((C_, S, 3))
    vel[..., 0] = 0.05 + 0.01 * np.sin(np.arange(S) / 5.0)[None, :]
    vel[..., 1] = rng.normal(0.0, 0.01, (C_, 1))
    yaw = rng.normal(0, 0.02, C_)
    att = np.stack([np.cos(yaw / 2), 0 * yaw, 0 * yaw, np.sin(yaw / 2)], 1)
    cases["persample"] = dict(raw=sc.raw, sample_times=sc.radar.sample_times(), pos=pos.astype(np.float32),
                              vel=vel.astype(np.float32), att=per_sample(att, C_, S),
                              grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                              start_freq=np.float32(sc.radar.f0), center=2.0, bw=20.0, centroid=1,
                              apply_range_win=1, taper=1, bore=np.array([0, 1, 0], np.float32))
    # E: non-uniform (jittered) sample times, infinite Doppler band
    sc = scenes.small_scene(seed=107, n_pri=160, n_samples=56, nx=10, ny=8, jitter=0.2e-3, device="cuda")
    st = sc.radar.sample_times().astype(np.float64)
    st += np.random.default_rng(108).uniform(-0.3, 0.3, st.shape) * (st[1] - st[0])
    cases["nonuniform"] = dict(raw=sc.raw, sample_times=st.astype(np.float32), pos=sc.positions.astype(np.float32),
                               vel=np.zeros((160, 3), np.float32),
                               att=np.tile([1, 0, 0, 0], (160, 1)).astype(np.float32),
                               grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                               start_freq=np.float32(sc.radar.f0), center=0.0, bw=float("inf"), centroid=0,
                               apply_range_win=1, taper=1, bore=np.array([0, 1, 0], np.float32))
    # F: one sample per chirp, 130 PRIs (a last chunk of two rows, the rest stale), moving
    # antenna, centroid window with taper
    rng = np.random.default_rng(109)
    sc = scenes.small_scene(seed=110, n_pri=130, n_samples=1, nx=9, ny=7, rail_len=0.2, device="cuda")
    vel = np.zeros((130, 3), np.float32)
    vel[:, 0] = 0.06
    yaw = rng.normal(0, 0.03, 130)
    att = np.stack([np.cos(yaw / 2), 0 * yaw, 0 * yaw, np.sin(yaw / 2)], 1).astype(np.float32)
    # (a one-sample Hann window is zero: seeded complex Gaussian samples instead)
    raw1 = (rng.normal(size=(130, 1)) + 1j * rng.normal(size=(130, 1))).astype(np.complex64)
    cases["onesample"] = dict(raw=raw1, sample_times=sc.radar.sample_times(), pos=sc.positions.astype(np.float32),
                              vel=vel, att=att, grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                              start_freq=np.float32(sc.radar.f0), center=1.0, bw=22.0, centroid=1,
                              apply_range_win=1, taper=1, bore=np.array([0, 1, 0], np.float32))
    # G: 17 samples per chirp (odd, not a multiple of the engine's 8-sample blocks), 75 PRIs
    # (a single partial chunk), reference range window, rectangular window, fixed centre
    sc = scenes.small_scene(seed=111, n_pri=75, n_samples=17, nx=11, ny=6, rail_len=0.15, device="cuda")
    vel = np.zeros((75, 3), np.float32)
    vel[:, 0] = 0.03
    cases["odd"] = dict(raw=sc.raw, sample_times=sc.radar.sample_times(), pos=sc.positions.astype(np.float32),
                        vel=vel, att=np.tile([1, 0, 0, 0], (75, 1)).astype(np.float32),
                        grid=sc.grid.astype(np.float32), mod_rate=np.float32(sc.radar.mod_rate),
                        start_freq=np.float32(sc.radar.f0), center=-1.0, bw=16.0, centroid=0, apply_range_win=1,
                        taper=0, bore=np.array([0, 1, 0], np.float32))
    return cases


def main() -> int:
    from oracle import build as ob

    ptx_path = ob.build_ref_ptx()
    if ptx_path is None or not Path(ptx_path).exists():
        print("oracle/_ref/tdckernels.ptx is missing: build it next to the reference checkout first")
        return 1
    drv = Driver(Path(ptx_path).read_bytes())
    cases = make_cases()
    flat = {}
    for name, case in cases.items():
        img = reference_focus(drv, case)
        for k, v in case.items():
            flat[f"{name}__{k}"] = np.asarray(v)
        flat[f"{name}__image"] = img
        print(name, "peak", float(np.abs(img).max()))
    np.savez_compressed(OUT, **flat)
    print("wrote", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
