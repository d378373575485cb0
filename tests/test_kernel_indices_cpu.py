"""CPU checks of the index arithmetic of the anchored-range focus kernel and of the work-unit
spans, against the constants of csrc/tdc_internal.h (no GPU: the formulas restated here are
the ones tdc_focus.cu and tdc_capi.cpp use)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
INTERNAL = (ROOT / "sarlab-tdc_gb300" / "csrc" / "tdc_internal.h").read_text()


def _const(name):
    m = re.search(rf"constexpr int {name} = ([^;]+);", INTERNAL)
    assert m, name
    return m.group(1).strip()


def _focus_geometry():
    pt = int(re.search(r"#define TDC_FOCUS_PT (\d+)", INTERNAL).group(1))
    threads = int(_const("kFocusThreads"))
    max_chirps = int(_const("kAnchorMaxStageChirps"))
    return pt, threads, max_chirps


def test_anchor_records_and_anchors_stay_in_their_buffers():
    """Per stage, record k = chirp x slots + slot for k < slots x chirps: within the shared buffer
    of slots x kAnchorMaxStageChirps records per warp, reading the stage's own chirp record and
    its warp's anchor; each slot's anchor is a pixel of its 32 (the 17th, or the last inside the
    grid) for every grid end."""
    pt, threads, max_chirps = _focus_geometry()
    recs_per_warp = pt * max_chirps
    tile = threads * pt
    for cb in range(1, max_chirps + 1):
        for cnt in range(1, cb + 1):
            for k in range(pt * cnt):
                assert k < recs_per_warp
                assert (k >> 2) < cnt and (k & (pt - 1)) < pt and k == (k >> 2) * pt + (k & (pt - 1))
    for P in (1, 31, 32, 33, 511, 512, 513, 1000, 1083):
        for t in range((P + tile - 1) // tile):
            for warp in range(threads // 32):
                for i in range(pt):
                    base = t * tile + i * threads + warp * 32
                    n_valid = min(32, P - base)
                    if n_valid > 0:
                        a = base + min(16, n_valid - 1)
                        assert base <= a < min(P, base + 32)


def test_kernel_rejects_stages_beyond_its_anchor_records():
    """The kernel's guard (slots x stage chirps > records per warp: report, no copy) fires exactly
    above kAnchorMaxStageChirps, the host's own limit."""
    pt, _, max_chirps = _focus_geometry()
    assert all((pt * cb > pt * max_chirps) == (cb > max_chirps) for cb in range(1, 4 * max_chirps))


def test_unit_span_encoding_round_trips():
    """FocusUnit::span: marker bit, 15-bit offsets lo and hi within the chirp group; 0 means the
    whole group, and an empty span still carries the marker."""
    m = re.fullmatch(r"1 << (\d+)", _const("kUnitSpanMax"))
    assert m
    span_max = 1 << int(m.group(1))
    assert span_max == 1 << 15

    def enc(lo, hi):
        return (1 << 30) | (lo << 15) | hi

    for lo, hi in ((0, 0), (0, 1), (5, 9), (0, span_max - 1), (span_max - 1, span_max - 1)):
        s = enc(lo, hi)
        assert s != 0 and (s >> 15) & (span_max - 1) == lo and s & (span_max - 1) == hi
        assert 0 < s < 2 ** 31
