"""Generate the golden vectors under tests/golden/ from the reference itself.

Run in a checkout next to the sarlab-tdc reference (``TDC_REFERENCE_ROOT``,
default /root/reference):

    python tests/golden/make_golden.py

It builds ``oracle/_ref/libtdc_refmath.so`` -- the reference's own
``tdc-lib/include/gpumath.h`` and ``windowing.h`` compiled for the host (see
oracle/build.py) -- and records:

* ``mathtest_known_answers.json``: the reference's function outputs at the
  inputs of its own unit tests (tdctest/mathtest.cpp), next to the expected
  values those tests assert;
* ``refmath_vectors.json``: outputs of the same reference functions at seeded
  random inputs (trajectory, attitude and Doppler-window values of the kind the
  focus path evaluates), the fixture the oracle is pinned to in CPU tests;
* ``reference_constants.json``: PRI_CHUNKSIZE and the window ``a`` parameters
  (tuning.h:18,31,38) as compiled.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build as obuild  # noqa: E402

OUT = Path(__file__).resolve().parent
F = C.POINTER(C.c_float)


def fa(v):
    return (C.c_float * len(v))(*[float(x) for x in v])


def main() -> int:
    path = obuild.build_refmath(force=True)
    if path is None:
        print("reference checkout not found; golden vectors not regenerated")
        return 1
    from oracle import refmath
    R = refmath()

    def q_prod(a, b):
        o = (C.c_float * 4)()
        R.ref_q_prod(fa(a), fa(b), o)
        return list(o)

    def q_rot(q, v):
        o = (C.c_float * 3)()
        R.ref_q_rot(fa(q), fa(v), o)
        return list(o)

    def q_conj(q):
        o = (C.c_float * 4)()
        R.ref_q_conj(fa(q), o)
        return list(o)

    def add2(a, b):
        o = (C.c_float * 2)()
        R.ref_float2_add(fa(a), fa(b), o)
        return list(o)

    def sub3(a, b):
        o = (C.c_float * 3)()
        R.ref_float3_sub(fa(a), fa(b), o)
        return list(o)

    # ---- known answers at the inputs of tdctest/mathtest.cpp ----
    h = math.sqrt(2.0) / 2.0
    ka = {
        "source": "tdctest/mathtest.cpp",
        "norm3df": {"in": [2, 4, 6], "ref": R.ref_norm3(2.0, 4.0, 6.0), "expect": math.sqrt(56.0),
                    "cite": "mathtest.cpp:12-19"},
        "float2_add": [
            {"a": a, "b": b, "ref": add2(a, b), "expect": [a[0] + b[0], a[1] + b[1]]}
            for a, b in [([1, 2], [3, 5]), ([1, 2], [-3, -5]), ([0, 0], [1, 1]), ([1, 1], [0, 0])]],
        "float3_sub": [
            {"a": a, "b": b, "ref": sub3(a, b), "expect": [a[i] - b[i] for i in range(3)]}
            for a, b in [([1, 2, 3], [4, 8, 12]), ([1, 2, 3], [-4, -8, -12]), ([1, 1, 1], [0, 0, 0]),
                         ([0, 0, 0], [1, 1, 1])]],
        "v3_dot": [
            {"a": a, "b": [4, 8, 12], "ref": R.ref_dot3(fa(a), fa([4, 8, 12])), "expect": e}
            for a, e in [([1, 0, 0], 4), ([0, 1, 0], 8), ([0, 0, 1], 12), ([1, 1, 1], 24)]],
        "q_conj": {"in": [1, 2, 3, 4], "ref": q_conj([1, 2, 3, 4]), "expect": [1, -2, -3, -4],
                   "cite": "mathtest.cpp:102-110"},
        "q_prod": {"a": [1, 2, 3, 4], "b": [8, 7, 6, 5], "ref": q_prod([1, 2, 3, 4], [8, 7, 6, 5]),
                   "expect": [-44, 14, 48, 28], "cite": "mathtest.cpp:112-121"},
        "q_rot": [
            {"q": [h, 0, 0, h], "v": [1, 0, 0], "ref": q_rot([h, 0, 0, h], [1, 0, 0]), "expect": [0, 1, 0],
             "cite": "mathtest.cpp:126-130"},
            {"q": [h, 0, 0, -h], "v": [1, 0, 0], "ref": q_rot([h, 0, 0, -h], [1, 0, 0]), "expect": [0, -1, 0],
             "cite": "mathtest.cpp:132-136"},
        ],
    }
    (OUT / "mathtest_known_answers.json").write_text(json.dumps(ka, indent=1))

    # ---- seeded vectors over the window math ----
    rng = np.random.default_rng(20261203)
    n = 64
    vecs = []
    for _ in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        q = q.astype(np.float32)
        bore = rng.normal(size=3).astype(np.float32)
        bore /= np.float32(np.linalg.norm(bore))
        vel = rng.normal(0, 0.5, 3).astype(np.float32)
        pos = (rng.normal(size=3) * [0.5, 0.1, 0.3] + [0, 0, 0.3]).astype(np.float32)
        tgt = (rng.normal(size=3) * [0.3, 0.3, 0.02] + [0, 0.4, 0]).astype(np.float32)
        lam = np.float32(299792458.0 / 79e9)
        ant = q_rot(q, bore)
        fdc = R.ref_doppler_centroid(fa(vel), fa(ant), lam)
        fd = R.ref_doppler_freq(fa(pos), fa(vel), fa(tgt), lam)
        bw = np.float32(abs(rng.normal(0, 8.0)) + 0.5)
        centre = np.float32(rng.normal(0, 3.0))
        vecs.append({
            "q": q.tolist(), "bore": bore.tolist(), "vel": vel.tolist(), "pos": pos.tolist(), "tgt": tgt.tolist(),
            "lambda": float(lam), "bw": float(bw), "centre": float(centre),
            "q_rot": ant, "doppler_centroid": fdc, "doppler_freq": fd,
            "window_taper": R.ref_doppler_window(fd, centre, bw, 1),
            "window_rect": R.ref_doppler_window(fd, centre, bw, 0),
        })
    (OUT / "refmath_vectors.json").write_text(json.dumps({"source": "tdc-lib/include/gpumath.h, windowing.h",
                                                           "vectors": vecs}, indent=1))
    consts = {"PRI_CHUNKSIZE": R.ref_pri_chunksize(), "RANGE_WINDOW_A_PARAMETER": R.ref_range_window_a(),
              "AZIMUTH_WINDOW_A_PARAMETER": R.ref_azimuth_window_a(), "source": "tdc-lib/include/tuning.h"}
    (OUT / "reference_constants.json").write_text(json.dumps(consts, indent=1))
    print("wrote golden vectors to", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
